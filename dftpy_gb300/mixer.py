"""Density mixers of OE-SCF (src/dftpy/mixer/__init__.py:5-52, mixer.py:8-169,
pulay.py:8-120, linear.py:4-35).

Fields and the Pulay history stay on the device; each mixing step is one
history kernel, one Gram-matrix pass over the history (the Pulay matrix and
right-hand side together), a host solve of the small symmetric system, and
one preconditioned combination (real-space combination, batched R2C, G-space
matrix, C2R) in the native library.
"""
import numpy as np
import torch
from scipy import linalg

from . import _lib
from .field import DirectField
from .functional.abstract_functional import stream_ptr

__all__ = ["Mixer", "PulayMixer", "LinearMixer", "SpecialPrecondition", "AbstractMixer"]

_PRED = {None: _lib.PRED_NONE, "kerker": _lib.PRED_KERKER, "inverse_kerker": _lib.PRED_INVERSE_KERKER,
         "resta": _lib.PRED_RESTA}


def _ptr(t):
    return _lib.C.c_void_p(t.data_ptr())


def _raw(f):
    t = f.as_subclass(torch.Tensor) if isinstance(f, torch.Tensor) else torch.as_tensor(f)
    return t.contiguous()


def _field(grid, t):
    out = t.as_subclass(DirectField)
    out.grid = grid
    out._N = None
    return out


class SpecialPrecondition:
    """The G-space preconditioner of the mixed residual (mixer.py:8-151):
    None (1), 'kerker' a0 min(G^2/(G^2 + q0^2), amin), 'inverse_kerker'
    b0^2/G^2 + 1 (0 at G = 0), 'resta'; with predecut, linear mixing above the
    cutoff."""

    def __init__(self, predtype="inverse_kerker", predcoef=[0.8, 1.0, 1.0], grid=None, predecut=None, **kwargs):
        if predtype not in _PRED:
            raise AttributeError("!!!ERROR : NOT support predtype %r" % (predtype,))
        self.predtype = predtype
        self.predcoef = self._init_predcoef(predcoef)
        self._ecut = predecut
        self._grid = grid

    @staticmethod
    def _init_predcoef(predcoef):
        pc = [float(x) for x in (predcoef or [])]
        if len(pc) == 0:
            pc = [0.8, 1.0, 1.0]
        while len(pc) < 3:
            pc.append(1.0)
        return pc

    @property
    def grid(self):
        return self._grid

    @grid.setter
    def grid(self, value):
        self._grid = value

    def args(self, coef, mask_coef, resw=1.0):
        a = _lib.MixArgs()
        a.predtype = _PRED[self.predtype]
        for k in range(3):
            a.predcoef[k] = self.predcoef[k]
        a.cutoff = 0 if self._ecut is None else 1
        a.predecut = 0.0 if self._ecut is None else float(self._ecut)
        a.coef, a.mask_coef, a.resw = float(coef), float(mask_coef), float(resw)
        a.ns = 0
        return a

    def run(self, nin, nout, a):
        """The native preconditioned combination of nin, nout and the history in a."""
        if self.grid is None:
            self.grid = nin.grid
        grid = nin.grid
        tin, tout = _raw(nin), _raw(nout)
        out = torch.empty_like(tin)
        _lib.check(_lib.load().ofdft_mix_density(grid.native_for(tin.dtype), _ptr(tin), _ptr(tout),
                                                 _lib.C.byref(a), _ptr(out), stream_ptr()))
        return _field(grid, out)

    def __call__(self, nin, nout, drho=None, residual=None, coef=0.7):
        return self.compute(nin, nout, drho, residual, coef)

    def compute(self, nin, nout, drho=None, residual=None, coef=0.7):
        """mixer.py:126-140: IFFT(FFT(nin) + FFT(drho) + M FFT(residual)), and the
        linear mix of nin and nout (weight coef) above the cutoff."""
        a = self.args(coef=1.0, mask_coef=coef, resw=0.0)
        keep = []
        if drho is not None or residual is not None:
            a.ns = 1
            a.x[0] = 1.0
            if drho is not None:
                t = _raw(drho)
                keep.append(t)
                a.dn[0] = t.data_ptr()
            if residual is not None:
                t = _raw(residual)
                keep.append(t)
                a.dr[0] = t.data_ptr()
        return self.run(nin, nout, a)


class AbstractMixer:
    """mixer.py:154-169."""

    def restart(self, *arg, **kwargs):
        pass

    def format_density(self, results, nin):
        # normalization_density(..., method='no') (density.py:319-337) leaves the density as it is
        return results


class PulayMixer(AbstractMixer):
    """pulay.py:8-120: Pulay (DIIS) mixing, G. Kresse and J. Furthmueller,
    Comput. Mat. Sci. 6, 15-50 (1996), with a history of at most maxm steps."""

    def __init__(self, predtype=None, predcoef=[0.8, 1.0, 1.0], maxm=5, coef=0.7, delay=0, predecut=None,
                 restarted=False, **kwargs):
        if maxm > _lib.MIX_MAXM:
            raise NotImplementedError("Pulay history of %d steps (at most %d)" % (maxm, _lib.MIX_MAXM))
        self.pred = SpecialPrecondition(predtype, predcoef, predecut=predecut)
        self._delay = delay
        self.maxm = int(maxm)
        self.coef = coef
        self.restarted = restarted
        self.restart()

    def __call__(self, nin, nout, coef=None):
        return self.compute(nin, nout, coef)

    def restart(self):
        self._iter = 0
        self._slots = []       # (dn, dr) device fields, oldest first
        self._free = []
        self._prev = None      # (density, residual) of the last step

    def residual(self, nin, nout):
        return nout - nin

    def _history_step(self, nin, nout, first):
        tin, tout = _raw(nin), _raw(nout)
        if self._prev is None or self._prev[0].dtype != tin.dtype or self._prev[0].shape != tin.shape:
            self._prev = (torch.empty_like(tin), torch.empty_like(tin))
            self._slots, self._free = [], []
            first = True
        dn = dr = None
        if not first:
            if len(self._slots) >= self.maxm:
                dn, dr = self._slots.pop(0)
            elif self._free:
                dn, dr = self._free.pop()
            else:
                dn, dr = torch.empty_like(tin), torch.empty_like(tin)
        _lib.check(_lib.load().ofdft_mix_history(nin.grid.native_for(tin.dtype), _ptr(tin), _ptr(tout),
                                                 _ptr(self._prev[0]), _ptr(self._prev[1]),
                                                 _ptr(dn) if dn is not None else None,
                                                 _ptr(dr) if dr is not None else None, 1 if first else 0,
                                                 stream_ptr()))
        if not first:
            self._slots.append((dn, dr))

    def compute(self, nin, nout, coef=None):
        if coef is None:
            coef = self.coef
        self._iter += 1
        if self._iter == 1 and self._delay < 1:
            results = self.pred.run(nin, nout, self.pred.args(coef, 0.7))  # pred's default coef (mixer.py:123)
            self._history_step(nin, nout, first=True)
        elif self._iter > self._delay:
            if self.restarted and (self._iter - self._delay) % (self.maxm + 1) == 0:
                self._free.extend(self._slots)
                self._slots = []
            self._history_step(nin, nout, first=False)
            ns = len(self._slots)
            fields = [s[1] for s in self._slots] + [self._prev[1]]
            nf = ns + 1
            arr = (_lib.C.c_void_p * nf)(*[f.data_ptr() for f in fields])
            gram = np.zeros((nf, nf))
            _lib.check(_lib.load().ofdft_mix_gram(nin.grid.native_for(fields[0].dtype), arr, nf,
                                                  gram.ctypes.data_as(_lib._PD), stream_ptr()))
            amat = gram[:ns, :ns].copy()
            b = -gram[:ns, ns]
            try:
                x = linalg.solve(amat, b, assume_a="sym")
                a = self.pred.args(coef, coef)
                a.ns = ns
                for k, (dn, dr) in enumerate(self._slots):
                    a.dn[k], a.dr[k], a.x[k] = dn.data_ptr(), dr.data_ptr(), float(x[k])
                results = self.pred.run(nin, nout, a)
            except Exception:
                # pulay.py:93-98: linear mixing when the Pulay system cannot be solved
                results = self.pred.run(nin, nout, self.pred.args(coef, coef))
        else:
            results = _field(nin.grid, _raw(nout).clone())
            self._history_step(nin, nout, first=True)
        return self.format_density(results, nin)


class LinearMixer(AbstractMixer):
    """linear.py:4-35: nin + M (coef (nout - nin)) after `delay` steps of nout."""

    def __init__(self, predtype="inverse_kerker", predcoef=[0.8, 1.0, 1.0], coef=0.7, delay=0, predecut=None,
                 **kwargs):
        self.pred = SpecialPrecondition(predtype, predcoef, predecut=predecut)
        self.coef = coef
        self._delay = delay
        self.restart()

    def restart(self):
        self._iter = 0

    def __call__(self, nin, nout, coef=None):
        return self.compute(nin, nout, coef)

    def compute(self, nin, nout, coef=None):
        self._iter += 1
        one = 1.0 - 1e-10
        if coef is None:
            coef = self.coef
        if self._iter > self._delay and coef < one:
            results = self.pred.run(nin, nout, self.pred.args(coef, coef))
            results = self.format_density(results, nin)
        else:
            results = _field(nin.grid, _raw(nout).clone())
        return results

    def residual(self, nin, nout):
        return nout - nin


class Mixer:
    """mixer/__init__.py:5-52: Mixer(scheme='pulay'|'linear'|None, **kwargs);
    scheme None or 'none' gives None."""

    def __new__(cls, scheme=None, **kwargs):
        if not scheme or str(scheme).lower() == "none":
            return None
        return super().__new__(cls)

    def __init__(self, scheme=None, nspin=2, **kwargs):
        self.mixers = [self.get_mixer(scheme=scheme, **kwargs) for _ in range(nspin)]

    def get_mixer(self, scheme=None, **kwargs):
        scheme = (scheme or "none").lower()
        if scheme == "pulay":
            return PulayMixer(**kwargs)
        if scheme == "linear":
            return LinearMixer(**kwargs)
        if scheme == "none":
            return None
        raise AttributeError("!!!ERROR : NOT support %s" % scheme)

    def __call__(self, nin, nout, coef=None):
        return self.compute(nin, nout, coef)

    def compute(self, nin, nout, coef=None):
        if getattr(nin, "rank", 1) != 1:
            raise NotImplementedError("spin-polarised densities are not supported")
        return self.mixers[0](nin, nout, coef=coef)

    def restart(self, *args, **kwargs):
        for m in self.mixers:
            m.restart(*args, **kwargs)
