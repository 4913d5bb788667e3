"""Persistent batched E+V evaluation of many independent systems.

The reference evaluates one system per ``TotalFunctional.compute`` call
(src/dftpy/functional/total_functional.py:107-146); this module has no
counterpart there.  ``BatchEvaluator`` holds a batch of total functionals, each
on its own grid (uneven sizes allowed, one precision), and evaluates all their
energies and potentials in one cooperative launch of the native library
(``ofdft_batch_eval_*``): the pre-pass, the library's own mixed-radix
transforms, the Hartree and vW G-space factors and the post-pass of every
system, stage by stage.  The launch shape (threads per block, rows per row tile,
lines per column tile) comes from a project autotuner that times every
candidate shape on the batch itself; the chosen shapes can be saved to and
loaded from a JSON tuning table.

Eligible functionals: TF, vW (no smoothing), LDA, Hartree and the local
pseudopotential, the functional of a batch of small systems.
"""
import ctypes as C
import json
import os

import torch

from . import _lib
from .field import DirectField
from .functional.abstract_functional import stream_ptr
from .functional.functional_output import FunctionalOutput

__all__ = ["BatchEvaluator"]


class BatchEvaluator:
    """BatchEvaluator(functionals, grids, dtype=torch.float64, tune=True,
    tuning_table=None): one persistent evaluation of every system's E and V.

    ``tune``: time the candidate launch shapes on the first call (the fastest
    is kept for later batches of the same grids in this process).
    ``tuning_table``: a JSON file of shapes by batch signature; a stored shape
    is used instead of tuning, and a newly tuned one is written back."""

    def __init__(self, functionals, grids, dtype=torch.float64, tune=True, tuning_table=None):
        if len(functionals) != len(grids) or not functionals:
            raise ValueError("one grid per functional, at least one system")
        self.functionals = list(functionals)
        self.grids = list(grids)
        self.dtype = dtype
        self.tune = bool(tune)
        self.tuning_table = tuning_table
        self._evs = []
        for tot, g in zip(self.functionals, self.grids):
            ev = tot.evaluator(g, dtype)
            tot.prepare(ev, g, dtype)
            lib = _lib.load()
            if not lib.ofdft_batch_eval_eligible(ev.h):
                raise NotImplementedError("the batched evaluation takes TF, vW, LDA, Hartree and the local "
                                          "pseudopotential only, on axes that are products of 2, 3 and 5 up to 128")
            self._evs.append(ev)
        self._h = None
        self.shape = None

    @property
    def signature(self):
        return ("f64" if self.dtype == torch.float64 else "f32") + "".join(
            ":%dx%dx%d" % tuple(g.nr) for g in self.grids)

    def _ptrs(self, tensors):
        return (C.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])

    def _create(self, rhos, vs):
        lib = _lib.load()
        n = len(self._evs)
        evs = (C.c_void_p * n)(*[ev.h for ev in self._evs])
        stored = self._load_table().get(self.signature)
        h = C.c_void_p()
        tune = self.tune and stored is None
        _lib.check(lib.ofdft_batch_eval_create(n, evs, 1 if tune else 0, self._ptrs(rhos), self._ptrs(vs),
                                               stream_ptr(), C.byref(h)))
        self._h = h
        if stored is not None:
            _lib.check(lib.ofdft_batch_eval_set_shape(h, int(stored["block"]), int(stored["rows"]),
                                                      int(stored["lines"])))
        self.shape = self.launch_shape()
        if tune and self.tuning_table:
            table = self._load_table()
            table[self.signature] = {k: self.shape[k] for k in ("block", "rows", "lines", "tuned_ms")}
            with open(self.tuning_table, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)

    def _load_table(self):
        if not self.tuning_table or not os.path.exists(self.tuning_table):
            return {}
        with open(self.tuning_table) as f:
            return json.load(f)

    def launch_shape(self):
        lib = _lib.load()
        b, r, l, g = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        ms = C.c_double()
        _lib.check(lib.ofdft_batch_eval_shape(self._h, C.byref(b), C.byref(r), C.byref(l), C.byref(g),
                                              C.byref(ms)))
        return {"block": b.value, "rows": r.value, "lines": l.value, "grid": g.value, "tuned_ms": ms.value}

    def __call__(self, rhos, active=None, out=None):
        """E and V of every system (or of those with active[i] true): a list of
        FunctionalOutput (None for inactive systems)."""
        n = len(self._evs)
        rs = []
        for rho, g in zip(rhos, self.grids):
            t = rho.as_subclass(torch.Tensor) if isinstance(rho, DirectField) else torch.as_tensor(rho)
            rs.append(t.to(device="cuda", dtype=self.dtype).contiguous())
        vs = out if out is not None else [torch.empty_like(t) for t in rs]
        if self._h is None:
            self._create(rs, vs)
        act = None
        if active is not None:
            act = (C.c_ubyte * n)(*[1 if a else 0 for a in active])
        E = (C.c_double * (n * _lib.NE))()
        _lib.check(_lib.load().ofdft_batch_eval_run(self._h, self._ptrs(rs), self._ptrs(vs), act, E,
                                                    stream_ptr()))
        res = []
        for i, (v, g) in enumerate(zip(vs, self.grids)):
            if active is not None and not active[i]:
                res.append(None)
                continue
            vf = v.as_subclass(DirectField)
            vf.grid = g
            vf._N = None
            res.append(FunctionalOutput(name="TOTAL", energy=float(E[i * _lib.NE + _lib.E_TOTAL]), potential=vf))
        return res

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                _lib.load().ofdft_batch_eval_destroy(self._h)
            except Exception:
                pass
            self._h = None
