"""ExternalPotential (src/dftpy/functional/external_potential.py:7-40): a frozen
potential v, energy dV sum(v rho), potential v.  In a total functional it is
one more term of the fused native evaluation (ofdft_eval_set_external)."""
import torch

from .. import _lib
from ..field import DirectField
from .abstract_functional import NativeFunctional

__all__ = ["ExternalPotential"]


class ExternalPotential(NativeFunctional):
    energy_slot = _lib.E_EXT
    out_name = "ext"

    def __init__(self, v=None):
        self.name = "EXT"
        self.type = "EXT"
        self._v = v
        self._version = 0

    def __repr__(self):
        return "EXT"

    @property
    def v(self):
        return self._v

    @v.setter
    def v(self, new_v):
        self._v = new_v
        self._version += 1

    @property
    def grid(self):
        return getattr(self._v, "grid", None)

    def potential(self):
        return self.v

    def configure(self, cfg):
        cfg.external = 1

    def prepare(self, ev, grid, dtype):
        if self._v is None:
            raise AttributeError("ExternalPotential: no potential set")
        token = (id(self._v), self._version, dtype)
        if getattr(ev, "ext_token", None) == token:
            return
        t = self._v.as_subclass(torch.Tensor) if isinstance(self._v, torch.Tensor) else torch.as_tensor(self._v)
        t = t.to(device="cuda", dtype=dtype).contiguous()
        if t.numel() != grid.nnr:
            raise ValueError("ExternalPotential: the potential has %d points, the grid %d" % (t.numel(), grid.nnr))
        ev.set_external(t)
        ev.ext_token = token

    def compute(self, density, calcType={"E", "V"}, **kwargs):
        out = NativeFunctional.compute(self, density, calcType)
        if "V" in calcType and isinstance(self._v, DirectField) and self._v.dtype == density.dtype:
            out.potential = self._v  # the reference hands back v itself
        return out
