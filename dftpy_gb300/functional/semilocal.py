"""XC (built-in LDA, src/dftpy/functional/xc/__init__.py:9-69 and
xc/semilocal_xc.py:283-341) and Hartree (src/dftpy/functional/hartree.py:11-45)."""
import numpy as np

from .. import _lib
from .abstract_functional import NativeFunctional

__all__ = ["XC", "Hartree"]


class XC(NativeFunctional):
    """Exchange-correlation: the reference's built-in LDA (Slater exchange +
    Perdew-Zunger 81 correlation, unpolarised)."""

    energy_slot = _lib.E_TOTAL
    out_name = "XC"

    def __init__(self, xc=None, core_density=None, libxc=None, name=None, pseudo=None, **kwargs):
        xc = xc or name
        if not xc and not libxc:
            raise ValueError("Please give a 'xc' or 'libxc'.")
        if isinstance(libxc, (list, tuple, str)) and not xc:
            names = [libxc] if isinstance(libxc, str) else list(libxc)
            if sorted(n.lower() for n in names) == ["lda_c_pz", "lda_x"]:
                xc = "LDA"
        if not xc or xc.upper() != "LDA":
            raise NotImplementedError("only the built-in LDA is on the accelerated path (got %r)" % (xc or libxc))
        if core_density is not None:
            raise NotImplementedError("non-linear core corrections are not supported")
        self.type = "XC"
        self.name = "LDA"
        self.options = dict(kwargs)
        self.pseudo = pseudo
        self.energy = None

    def configure(self, cfg):
        cfg.xc_lda = 1

    def compute(self, density, calcType={"E", "V"}, **kwargs):
        out = NativeFunctional.compute(self, density, calcType)
        if "E" in calcType:
            self.energy = out.energy
        return out

    def absorb_energies(self, energies):
        self.energy = float(energies[_lib.E_XC])

    def forces(self, density, pseudo=None, **kwargs):
        """NLCC forces: zero without core densities (xc/__init__.py:71-78)."""
        return None

    def stress(self, density, pseudo=None, energy=None, **kwargs):
        """XC.stress (xc/__init__.py:80-95) with _LDAStress (semilocal_xc.py:343-346):
        (E - int v_xc rho dV)/V on the diagonal.  A given (nonzero) energy replaces
        the one computed on density, as in the reference."""
        E = None
        if energy:
            E = np.zeros(_lib.NE)
            E[_lib.E_XC] = energy
        return self._native_stress(density, E)[_lib.S_XC].copy()


class _ClassOrInstance:
    """A method that also works on the class, through one shared instance
    (Hartree.compute is a classmethod in hartree.py:22-45)."""

    def __init__(self, f):
        self.f = f

    def __get__(self, obj, cls):
        if obj is None:
            obj = cls.__dict__.get("_shared") or cls._make_shared()
        return self.f.__get__(obj, cls)


class Hartree(NativeFunctional):
    energy_slot = _lib.E_TOTAL
    out_name = "Hartree"
    _energy = None
    _shared = None

    @classmethod
    def _make_shared(cls):
        cls._shared = cls()
        return cls._shared

    def __init__(self, **kwargs):
        self.type = "HARTREE"
        self.name = "HARTREE"
        self.options = kwargs

    def __repr__(self):
        return "HARTREE"

    def configure(self, cfg):
        cfg.hartree = 1

    @_ClassOrInstance
    def compute(self, density, calcType={"E", "V"}, **kwargs):
        out = NativeFunctional.compute(self, density, calcType)
        if "E" in calcType:
            Hartree._energy = out.energy
        return out

    def absorb_energies(self, energies):
        Hartree._energy = float(energies[_lib.E_H])

    @property
    def energy(self):
        return self._energy

    def stress(self, density, **kwargs):
        """Hartree.stress (hartree.py:51-56) with HartreeFunctionalStress (:67-90): the
        energy is the one the class cached at its last energy evaluation, or computed
        on density when there is none."""
        E = None
        if Hartree._energy is not None:
            E = np.zeros(_lib.NE)
            E[_lib.E_H] = Hartree._energy
        return self._native_stress(density, E)[_lib.S_H].copy()
