"""The Wang-Govind-Carter kinetic functional with the two-body Fermi wave vector
xi_gamma(r, r') = ((k_F(r)^gamma + k_F(r')^gamma)/2)^(1/gamma) (Y. A. Wang,
N. Govind, E. A. Carter, Phys. Rev. B 60, 16350 (1999)), evaluated through the
paper's second-order Taylor expansion of the kernel about the Fermi wave vector
of the reference density rho0, on the Wang-Teter kernel of the reference
(src/dftpy/functional/kedf/kernel.py:325-334).  The reference has no
implementation of it; this is the device path (``ofdft_wgc_*``).

``Functional(type="KEDF", name="WGC-NL", gamma=2.7, alpha=..., beta=..., x=1,
rho0=None)`` is the nonlocal term alone; ``name="WGC"`` adds TF and vW, as
"WT" does for the Wang-Teter term.  Defaults: alpha = (5 + sqrt 5)/6,
beta = (5 - sqrt 5)/6, gamma = 2.7, rho0 = the mean density of each call.
These terms are evaluated beside the fused evaluator (a TotalFunctional sums
them), so the native optimiser, which needs a fused evaluator, does not take
them.
"""
import ctypes as C

import torch

from .. import _lib
from ..field import DirectField, as_field
from .abstract_functional import AbstractFunctional, calc_bits, stream_ptr
from .functional_output import FunctionalOutput

__all__ = ["WGCNL", "WGCKEDF"]

WGC_ALPHA = (5.0 + 5.0 ** 0.5) / 6.0
WGC_BETA = (5.0 - 5.0 ** 0.5) / 6.0


class WGCNL(AbstractFunctional):
    """The nonlocal WGC term on the device."""

    def __init__(self, alpha=WGC_ALPHA, beta=WGC_BETA, gamma=2.7, x=1.0, rho0=None, **kwargs):
        self.type = "KEDF"
        self.name = "WGC-NL"
        self.alpha, self.beta, self.gamma, self.x = float(alpha), float(beta), float(gamma), float(x)
        self.rho0 = rho0
        self._h = {}

    def _handle(self, grid, dtype):
        key = (id(grid), dtype)
        h = self._h.get(key)
        if h is None:
            lib = _lib.load()
            p = C.c_void_p()
            _lib.check(lib.ofdft_wgc_create(grid.native_for(dtype), self.alpha, self.beta, self.gamma, self.x,
                                            float(self.rho0) if self.rho0 else 0.0, C.byref(p)))
            h = _Handle(lib, p)
            self._h[key] = h
        return h.p

    def compute(self, density, calcType={"E", "V"}, **kwargs):
        rho = density if isinstance(density, DirectField) else as_field(getattr(self, "grid", None), density)
        calc = calc_bits(calcType)
        t = rho.as_subclass(torch.Tensor).contiguous()
        V = torch.empty_like(t) if calc & _lib.CALC_V else None
        E = C.c_double()
        _lib.check(_lib.load().ofdft_wgc_compute(self._handle(rho.grid, rho.dtype), C.c_void_p(t.data_ptr()),
                                                 C.c_void_p(V.data_ptr()) if V is not None else None, calc,
                                                 C.byref(E), stream_ptr()))
        out = FunctionalOutput(name=self.name, energy=float(E.value) if calc & _lib.CALC_E else 0.0)
        if V is not None:
            v = V.as_subclass(DirectField)
            v.grid = rho.grid
            v._N = None
            out.potential = v
        return out


class WGCKEDF(AbstractFunctional):
    """KEDF "WGC" (TF + vW + WGC-NL) or "WGC-NL", with the options of both."""

    def __init__(self, name="WGC", **kwargs):
        from .kedf import KEDF
        self.type = "KEDF"
        self.name = name.upper()
        nl = {k: kwargs[k] for k in ("alpha", "beta", "gamma", "x", "rho0") if k in kwargs}
        self.nl = WGCNL(**nl)
        self.local = None
        if self.name == "WGC":
            self.local = KEDF(name="TFVW", **{k: kwargs[k] for k in ("x", "y") if k in kwargs})

    def compute(self, density, calcType={"E", "V"}, split=False, **kwargs):
        parts = {}
        if self.local is not None:
            if split:
                parts.update(self.local.compute(density, calcType=calcType, split=True))
            else:
                parts["TFVW"] = self.local.compute(density, calcType=calcType)
        parts["WGC-NL"] = self.nl.compute(density, calcType=calcType)
        if split:
            return parts
        total = None
        for r in parts.values():
            total = r if total is None else total + r
        total.name = "KEDF"
        return total


class _Handle:
    def __init__(self, lib, p):
        self.lib, self.p = lib, p

    def __del__(self):
        try:
            self.lib.ofdft_wgc_destroy(self.p)
        except Exception:
            pass
