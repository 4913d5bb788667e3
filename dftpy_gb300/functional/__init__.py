"""Functional plugin API (src/dftpy/functional/__init__.py:11-51)."""
from .abstract_functional import AbstractFunctional
from .external_potential import ExternalPotential
from .functional_output import FunctionalOutput, ZeroFunctional
from .kedf import KEDF
from .pseudo import LocalPseudo, ReadPseudo, RECPOT, read_recpot, write_recpot
from .semilocal import XC, Hartree
from .total_functional import TotalFunctional

__all__ = ["Functional", "FunctionalOutput", "ZeroFunctional", "AbstractFunctional", "TotalFunctional", "KEDF", "XC",
           "Hartree", "ExternalPotential", "LocalPseudo", "ReadPseudo", "RECPOT", "read_recpot", "write_recpot",
           "FunctionalTypeDict"]

FunctionalTypeDict = {
    "KEDF": KEDF,
    "PSEUDO": LocalPseudo,
    "HARTREE": Hartree,
    "XC": XC,
    "EXT": ExternalPotential,
}


def Functional(type=None, optional_kwargs=None, **kwargs):
    """Functional(type='KEDF'|'XC'|'HARTREE'|'PSEUDO'|'EXT', **kwargs)."""
    type = type.upper()
    if optional_kwargs is not None:
        kwargs.update(optional_kwargs)
    try:
        cls = FunctionalTypeDict[type]
    except KeyError:
        raise AttributeError("Unknown functional type: {}.".format(type))
    name = str(kwargs.get("name") or kwargs.get("kedf") or "")
    if type == "KEDF" and name.upper() in ("WGC", "WGC-NL"):
        # the two-body WGC kernel, beside the fused evaluator (no reference counterpart)
        from .wgc import WGCKEDF
        kw = {k: v for k, v in kwargs.items() if k not in ("name", "kedf")}
        return WGCKEDF(name=name, **kw)
    return cls(**kwargs)
