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
    return cls(**kwargs)
