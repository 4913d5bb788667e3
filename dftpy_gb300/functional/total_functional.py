"""TotalFunctional (src/dftpy/functional/total_functional.py:5-174).

``compute`` fuses every functional into one native evaluation: one pre-pass
over rho, the forward transforms, one fused G-space pass, the inverse
transforms and one post-pass that writes the total potential.
"""
import numpy as np
import torch

from .. import _lib
from ..field import DirectField, as_field
from .abstract_functional import AbstractFunctional, NativeEval, NativeFunctional, calc_bits, config_key, \
    empty_config
from .functional_output import FunctionalOutput

__all__ = ["TotalFunctional"]


class TotalFunctional(AbstractFunctional):
    def __init__(self, ewald=None, **kwargs):
        self.funcDict = {k: v for k, v in kwargs.items() if v is not None}
        self.UpdateNameType()
        self._ewald = ewald
        self._evals = {}

    def __repr__(self):
        return self.funcDict.__repr__()

    def __getitem__(self, key):
        return self.funcDict[key]

    def __setitem__(self, key, value):
        self.funcDict[key] = value
        self.UpdateNameType()

    def UpdateNameType(self):
        self.name = ""
        self.type = ""
        for key, f in self.funcDict.items():
            if not isinstance(f, AbstractFunctional):
                raise TypeError("{} must be AbstractFunctional".format(key))
            setattr(self, key, f)
            self.name += f.name + " "
            self.type += f.type + " "
        self._evals = {}

    def UpdateFunctional(self, keysToRemove=[], newFuncDict={}):
        for key in keysToRemove:
            self.funcDict.pop(key, None)
        self.funcDict.update(newFuncDict)
        self.UpdateNameType()

    def Subset(self, keys):
        return TotalFunctional(**{k: self.funcDict[k] for k in keys})

    @property
    def ewald(self):
        if self._ewald is not None:
            return self._ewald
        for f in self.funcDict.values():
            if f.type == "PSEUDO":
                return f.get_ewald()
        return None

    # -------------------------------------------------------- fused path
    def _fusable(self):
        if not all(isinstance(f, NativeFunctional) for f in self.funcDict.values()):
            return False
        seen = 0
        for f in self.funcDict.values():
            cfg = empty_config()
            f.configure(cfg)
            bits = cfg.kedf_terms | (cfg.xc_lda << 8) | (cfg.hartree << 9) | (cfg.pseudo << 10) | (cfg.external << 11)
            if bits & seen:
                return False  # a term configured twice: evaluate separately and sum
            seen |= bits
        return True

    def evaluator(self, grid, dtype):
        """The fused native evaluator of this total functional on (grid, dtype)."""
        cfg = empty_config()
        for f in self.funcDict.values():
            f.configure(cfg)
        key = (id(grid), dtype, config_key(cfg))
        ev = self._evals.get(key)
        if ev is None:
            ev = NativeEval(grid, dtype, cfg)
            self._evals[key] = ev
        return ev

    def prepare(self, ev, grid, dtype, with_ewald=True):
        for f in self.funcDict.values():
            f.prepare(ev, grid, dtype)
        ew = self.ewald if with_ewald else None
        ev.set_ewald(ew.energy if ew is not None else 0.0)

    def finish(self, ev):
        for f in self.funcDict.values():
            f.finish(ev)

    def compute(self, rho, calcType={"E", "V"}, **kwargs):
        return self.get_energy_potential(rho, calcType=calcType, **kwargs)

    def Energy(self, rho, **kwargs):
        return self.compute(rho, calcType={"E"}).energy

    def get_energy_potential(self, rho, calcType={"E", "V"}, split=False, **kwargs):
        if not isinstance(rho, DirectField):
            grid = next((getattr(f, "grid", None) for f in self.funcDict.values() if getattr(f, "grid", None)), None)
            rho = as_field(grid, rho)
        if split or not self._fusable():
            return self._separate(rho, calcType, split)
        calc = calc_bits(calcType)
        ev = self.evaluator(rho.grid, rho.dtype)
        self.prepare(ev, rho.grid, rho.dtype)
        E, V = ev.compute(rho, calc)
        self.finish(ev)
        if calc & _lib.CALC_E:
            # what each functional's own energy evaluation leaves behind in the
            # reference (the Hartree class energy, the XC energy)
            for f in self.funcDict.values():
                f.absorb_energies(E)
        out = FunctionalOutput(name="TOTAL", energy=float(E[_lib.E_TOTAL]) if calc & _lib.CALC_E else 0.0)
        if V is not None:
            v = V.as_subclass(DirectField)
            v.grid = rho.grid
            v._N = None
            out.potential = v
        out.energies = {"TF": E[_lib.E_TF], "VW": E[_lib.E_VW], "NL": E[_lib.E_NL], "XC": E[_lib.E_XC],
                        "HARTREE": E[_lib.E_H], "PSEUDO": E[_lib.E_PP], "II": E[_lib.E_II], "EXT": E[_lib.E_EXT]}
        return out

    def _separate(self, rho, calcType, split):
        parts = {"TOTAL": FunctionalOutput(name="TOTAL", energy=0.0)}
        for key, f in self.funcDict.items():
            if split and f.type == "KEDF":
                res = f(rho, calcType=calcType, split=True)
                for k2, r in res.items():
                    k = "KEDF-" + k2.split("-")[-1]
                    parts[k] = r
                    parts["TOTAL"] = parts["TOTAL"] + r
            else:
                r = f(rho, calcType=calcType)
                if split:
                    parts[f.type] = r
                parts["TOTAL"] = parts["TOTAL"] + r
        ew = self.ewald
        if ew is not None:
            r = FunctionalOutput(name="II", energy=ew.energy)
            if split:
                parts["II"] = r
            parts["TOTAL"] = parts["TOTAL"] + r
        return parts if split else parts["TOTAL"]

    def get_forces(self, rho, ions=None, split=False, **kwargs):
        """total_functional.py:148-174: PP forces + Ewald forces (XC NLCC forces are zero)."""
        ew = self.ewald
        if ions is None:
            if ew is None:
                raise ValueError("Please provide ions for forces")
            ions = ew.ions
        forces = {"TOTAL": np.zeros((ions.nat, 3))}
        for key, f in self.funcDict.items():
            if hasattr(f, "forces"):
                fr = f.forces(rho)
                if fr is not None:
                    if split:
                        forces[key] = fr
                    forces["TOTAL"] = forces["TOTAL"] + fr
        if ew is not None:
            fr = ew.forces
            if split:
                forces["II"] = fr
            forces["TOTAL"] = forces["TOTAL"] + fr
        return forces if split else forces["TOTAL"]

    def get_stress(self, rho, split=False, **kwargs):
        """total_functional.py:176-208: KEDF terms under "KEDF-<engine>", the other
        functionals under their type, the Ewald stress under "II", and their sum
        under "TOTAL"."""
        stress = {"TOTAL": np.zeros((3, 3))}
        for key, func in self.funcDict.items():
            if func.type == "KEDF":
                results = func.stress(rho, split=True)
                for key2, v in results.items():
                    stress["TOTAL"] = stress["TOTAL"] + v
                    k = "KEDF-" + key2.split("-")[-1]
                    stress[k] = stress.get(k, 0.0) + v
            else:
                v = func.stress(rho)
                stress["TOTAL"] = stress["TOTAL"] + v
                stress[func.type] = v
        ew = self.ewald
        if ew is not None:
            stress["II"] = ew.stress
            stress["TOTAL"] = stress["TOTAL"] + stress["II"]
        T = stress["TOTAL"]
        for i in range(1, 3):
            for j in range(i - 1, -1, -1):
                T[i, j] = T[j, i]
        return stress if split else stress["TOTAL"]
