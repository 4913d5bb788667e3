"""AbstractFunctional (src/dftpy/functional/abstract_functional.py:12-44) and the
native-evaluator plumbing shared by every functional on the hot path.

A functional describes its part of an ``ofdft_config`` (``configure``) and
binds any per-grid data the native evaluator needs (``prepare``).  Calling a
functional alone runs an evaluator configured with that functional only;
``TotalFunctional`` fuses all of its functionals into one evaluator.
"""
from abc import ABC, abstractmethod

import numpy as np
import torch

from .. import _lib
from ..field import DirectField, as_field
from .functional_output import FunctionalOutput

__all__ = ["AbstractFunctional", "NativeEval", "NativeFunctional", "calc_bits"]


def calc_bits(calcType):
    calc = set(calcType)
    unsupported = calc - {"E", "V"}
    if unsupported:
        raise NotImplementedError("calcType %s is not on the accelerated path (E and V only)" % sorted(unsupported))
    bits = 0
    if "E" in calc:
        bits |= _lib.CALC_E
    if "V" in calc:
        bits |= _lib.CALC_V
    return bits


def stream_ptr():
    return _lib.C.c_void_p(torch.cuda.current_stream().cuda_stream)


class NativeEval:
    """One native ofdft_eval handle: a configured total functional on one grid/precision."""

    def __init__(self, grid, dtype, cfg):
        self.lib = _lib.load()
        self.grid, self.dtype, self.cfg = grid, dtype, cfg
        h = _lib.C.c_void_p()
        _lib.check(self.lib.ofdft_eval_create(grid.native_for(dtype), _lib.C.byref(cfg), _lib.C.byref(h)))
        self.h = h
        self.vloc_token = None
        self._E = np.zeros(_lib.NE, dtype=np.float64)

    def __del__(self):
        try:
            if self.h:
                self.lib.ofdft_eval_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def set_vloc(self, vloc, token):
        if self.vloc_token is token:
            return
        t = vloc.as_subclass(torch.Tensor).contiguous()
        _lib.check(self.lib.ofdft_eval_set_vloc(self.h, _lib.C.c_void_p(t.data_ptr()), stream_ptr()))
        self.vloc_token = token

    def set_external(self, v):
        """Copy a frozen external potential (device tensor of the evaluator dtype) in."""
        _lib.check(self.lib.ofdft_eval_set_external(self.h, _lib.C.c_void_p(v.data_ptr()), stream_ptr()))

    def set_lwt_table(self, table):
        """Kernel table of the k_F-node term (values at linspace(0, etamax, neta))."""
        t = np.ascontiguousarray(table, dtype=np.float64)
        _lib.check(self.lib.ofdft_eval_set_lwt_table(self.h, t.ctypes.data_as(_lib._PD), len(t)))
        self.lwt_table_set = True

    def set_ewald(self, energy):
        _lib.check(self.lib.ofdft_eval_set_ewald(self.h, float(energy)))

    def kfbounds(self):
        a, b = _lib.C.c_double(), _lib.C.c_double()
        _lib.check(self.lib.ofdft_eval_get_kfbounds(self.h, _lib.C.byref(a), _lib.C.byref(b)))
        return (None if np.isnan(a.value) else a.value), (None if np.isnan(b.value) else b.value)

    def set_kfbounds(self, kfmin, kfmax):
        _lib.check(self.lib.ofdft_eval_set_kfbounds(self.h, np.nan if kfmin is None else float(kfmin),
                                                    np.nan if kfmax is None else float(kfmax)))

    def stats(self):
        n, l = _lib.C.c_int(), _lib.C.c_int()
        _lib.check(self.lib.ofdft_eval_last_stats(self.h, _lib.C.byref(n), _lib.C.byref(l)))
        return n.value, l.value

    def compute(self, rho, calc, out=None):
        """rho: contiguous device tensor of the evaluator dtype.  Returns (energies, V)."""
        r = rho.as_subclass(torch.Tensor) if isinstance(rho, torch.Tensor) else rho
        if not r.is_contiguous():
            r = r.contiguous()
        V = None
        if calc & _lib.CALC_V:
            V = out if out is not None else torch.empty_like(r)
        E = self._E
        _lib.check(self.lib.ofdft_eval_compute(self.h, _lib.C.c_void_p(r.data_ptr()),
                                               _lib.C.c_void_p(V.data_ptr()) if V is not None else None, calc,
                                               E.ctypes.data_as(_lib._PD), stream_ptr()))
        return E.copy(), V


    def stress(self, rho, energies=None):
        """Stress tensors of the evaluator's terms, (NS, 3, 3) Ha/Bohr^3 (ofdft_eval_stress).
        energies: array of NE term energies for the diagonal, or None to compute them on rho."""
        r = rho.as_subclass(torch.Tensor) if isinstance(rho, torch.Tensor) else rho
        if not r.is_contiguous():
            r = r.contiguous()
        S = np.zeros((_lib.NS, 3, 3))
        e = None
        if energies is not None:
            e = np.ascontiguousarray(energies, dtype=np.float64)
            if e.shape != (_lib.NE,):
                raise ValueError("energies must hold %d values" % _lib.NE)
        _lib.check(self.lib.ofdft_eval_stress(self.h, _lib.C.c_void_p(r.data_ptr()),
                                              e.ctypes.data_as(_lib._PD) if e is not None else None,
                                              S.ctypes.data_as(_lib._PD), stream_ptr()))
        return S


class AbstractFunctional(ABC):
    def __repr__(self):
        return getattr(self, "name", self.__class__.__name__)

    def __call__(self, rho, *args, **kwargs):
        return self.compute(rho, *args, **kwargs)

    @abstractmethod
    def compute(self, rho, *args, **kwargs):
        pass

    @property
    def name(self):
        if getattr(self, "_name", None) is None:
            self._name = self.type
        return self._name

    @name.setter
    def name(self, value):
        self._name = value

    @property
    def type(self):
        if getattr(self, "_type", None) is None:
            self._type = self.__class__.__name__
        return self._type

    @type.setter
    def type(self, value):
        self._type = value


def empty_config():
    cfg = _lib.Config()
    _lib.check(_lib.load().ofdft_config_init(_lib.C.byref(cfg), _lib.C.sizeof(cfg)))
    cfg.kedf_terms = 0
    cfg.xc_lda = 0
    cfg.hartree = 0
    cfg.pseudo = 0
    return cfg


def config_key(cfg):
    def key(v):
        if isinstance(v, float):
            return "nan" if np.isnan(v) else v
        if hasattr(v, "_length_"):  # ctypes array field
            return tuple(v)
        return v
    return tuple(key(getattr(cfg, f)) for f, _ in cfg._fields_)


class NativeFunctional(AbstractFunctional):
    """A functional evaluated by the native library."""

    energy_slot = _lib.E_TOTAL
    out_name = "FUNC"

    def configure(self, cfg):  # fill this functional's part of the evaluator config
        raise NotImplementedError

    def prepare(self, ev, grid, dtype):  # bind per-grid data (v_loc, k_F state) before a compute
        pass

    def finish(self, ev):  # read back state after a compute
        pass

    def absorb_energies(self, energies):  # state a functional keeps from an energy evaluation
        pass

    def _evaluator(self, grid, dtype):
        cache = self.__dict__.setdefault("_evals", {})
        cfg = empty_config()
        self.configure(cfg)
        key = (id(grid), dtype, config_key(cfg))
        ev = cache.get(key)
        if ev is None:
            ev = NativeEval(grid, dtype, cfg)
            cache[key] = ev
        return ev

    def compute(self, density, calcType={"E", "V"}, **kwargs):
        rho = density if isinstance(density, DirectField) else as_field(self._grid_of(density), density)
        grid = rho.grid
        calc = calc_bits(calcType)
        ev = self._evaluator(grid, rho.dtype)
        self.prepare(ev, grid, rho.dtype)
        E, V = ev.compute(rho, calc)
        self.finish(ev)
        out = FunctionalOutput(name=self.out_name)
        if calc & _lib.CALC_E:
            out.energy = float(E[self.energy_slot])
        else:
            out.energy = 0.0
        if V is not None:
            v = V.as_subclass(DirectField)
            v.grid = grid
            v._N = None
            out.potential = v
        return out

    def _native_stress(self, density, energies=None):
        """(NS, 3, 3) stress tensors of this functional's terms on density."""
        rho = density if isinstance(density, DirectField) else as_field(self._grid_of(density), density)
        ev = self._evaluator(rho.grid, rho.dtype)
        self.prepare(ev, rho.grid, rho.dtype)
        return ev.stress(rho, energies)

    def _grid_of(self, density):
        g = getattr(density, "grid", None) or getattr(self, "grid", None)
        if g is None:
            raise TypeError("density must be a DirectField (or the functional must know its grid)")
        return g
