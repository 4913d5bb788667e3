"""Ewald ion-ion energy, forces and stress (src/dftpy/ewald.py:197-968) on the device.

Sums are float64 in both precisions.  The real-space part is the exact image
sum within the reference's cutoff, taken over a cell list; the reciprocal part
is smooth PME (B-spline order ``BsplineOrder``) or the exact structure factor.
"""
import numpy as np

from . import _lib
from .ions import as_ions

__all__ = ["ewald"]


class ewald:
    def __init__(self, precision=1.0e-8, ions=None, rho=None, grid=None, verbose=False, BsplineOrder=10, PME=False,
                 Bspline=None, **kwargs):
        if ions is None:
            raise AttributeError("Must pass ions to Ewald")
        self.ions = as_ions(ions)
        if grid is None:
            if rho is None:
                raise AttributeError("Must pass grid or rho to Ewald")
            grid = rho.grid
        self.grid = grid.get_direct() if hasattr(grid, "get_direct") else grid
        self.precision = precision
        self.verbose = verbose
        self.order = BsplineOrder
        self.PME = PME
        self._parts = None
        self._forces = None
        self._stress = None

    def _run(self, want_forces):
        lib = _lib.load()
        pos = np.ascontiguousarray(self.ions.positions, dtype=np.float64)
        q = np.ascontiguousarray(self.ions.charges, dtype=np.float64)
        out = np.zeros(4)
        eta = _lib.C.c_double()
        F = np.zeros((len(q), 3)) if want_forces else None
        _lib.check(lib.ofdft_ewald(self.grid.native(_lib.F64), len(q), _lib.dptr(pos), _lib.dptr(q),
                                   float(self.precision), 1 if self.PME else 0, int(self.order), _lib.dptr(out),
                                   _lib.dptr(F) if F is not None else None, _lib.C.byref(eta), None))
        self._parts = out
        self.eta = eta.value
        if F is not None:
            self._forces = F

    @property
    def energy(self):
        if self._parts is None:
            self._run(False)
        return float(self._parts[0])

    def Energy_real(self):
        self.energy
        return float(self._parts[1])

    Energy_real_fast2 = Energy_real

    def Energy_rec(self):
        self.energy
        return float(self._parts[2])

    Energy_rec_PME = Energy_rec

    def Energy_corr(self):
        self.energy
        return float(self._parts[3])

    @property
    def forces(self):
        if self._forces is None:
            self._run(True)
        return self._forces

    @property
    def stress(self):
        """ewald.stress (:523-538): Stress_real + Stress_rec_PME or Stress_rec, 3x3 Ha/Bohr^3."""
        if self._stress is None:
            lib = _lib.load()
            pos = np.ascontiguousarray(self.ions.positions, dtype=np.float64)
            q = np.ascontiguousarray(self.ions.charges, dtype=np.float64)
            S = np.zeros((3, 3))
            eta = _lib.C.c_double()
            _lib.check(lib.ofdft_ewald_stress(self.grid.native(_lib.F64), len(q), _lib.dptr(pos), _lib.dptr(q),
                                              float(self.precision), 1 if self.PME else 0, int(self.order),
                                              _lib.dptr(S), _lib.C.byref(eta), None))
            self.eta = eta.value
            self._stress = S
        return self._stress

    def compute(self, *args, calcType={"E"}, **kwargs):
        from .functional.functional_output import FunctionalOutput
        return FunctionalOutput(name="Ewald", energy=self.energy)

    __call__ = compute
