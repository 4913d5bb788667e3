"""Density optimisation (src/dftpy/optimization/optimization.py:31-547).

``Optimization.optimize_rho`` runs entirely in the native library: the
direction (TN finite-difference Hessian CG, L-BFGS two-loop or CG-HS), the
norm-conserving rotation phi cos(theta) + p sin(theta), the MINPACK-2 line
search and every field operation stay on the device; only scalars cross to
the host.
"""
import math

import numpy as np
import torch

from . import _lib
from .field import DirectField, as_field
from .functional.abstract_functional import NativeFunctional, stream_ptr
from .functional.functional_output import FunctionalOutput
from .functional.total_functional import TotalFunctional

__all__ = ["Optimization", "optimize_rho_batch", "OESCF"]

# get_direction (optimization.py:179-203): "CG" is CG-HS; any other "CG-*" name falls
# to get_direction_CG's last branch, Fletcher-Reeves (math_utils.py:345-346)
_METHODS = {"TN": _lib.OPT_TN, "LBFGS": _lib.OPT_LBFGS, "CG-HS": _lib.OPT_CGHS, "CG": _lib.OPT_CGHS,
            "CG-PR": _lib.OPT_CGPR, "CG-DY": _lib.OPT_CGDY, "CG-CD": _lib.OPT_CGCD, "CG-LS": _lib.OPT_CGLS,
            "CG-FR": _lib.OPT_CGFR, "GD": _lib.OPT_GD, "DIIS": _lib.OPT_DIIS}


class Optimization:
    def __init__(self, optimization_method="CG-HS", optimization_options=None, EnergyEvaluator=None, guess_rho=None):
        self.rho = guess_rho
        self.optimization_options = dict(optimization_options or {})
        defaults = {"maxcor": 6, "ftol": 1.0e-7, "xtol": 1.0e-12, "maxfun": 50, "maxiter": 200, "maxls": 30,
                    "econv": 1.0e-5, "c1": 1e-4, "c2": 0.2, "algorithm": "EMM", "vector": "Orthogonalization",
                    "ncheck": 2, "h0": 1.0, "pconv": None, "linesearch": "wolfe", "linesearch_start": "reference"}
        for k, v in defaults.items():
            self.optimization_options.setdefault(k, v)
        if EnergyEvaluator is None:
            raise AttributeError("Must provide an energy evaluator")
        self.EnergyEvaluator = EnergyEvaluator
        # unknown names fail where the reference's get_direction does, in optimize_rho
        self._method_code = _METHODS.get(optimization_method,
                                         _lib.OPT_CGFR if str(optimization_method).startswith("CG") else None)
        o = self.optimization_options
        if o["algorithm"] != "EMM" or o["vector"] != "Orthogonalization":
            raise NotImplementedError("only algorithm='EMM' with vector='Orthogonalization' is supported")
        self.optimization_method = optimization_method
        self.verbose = False
        self.mu = None
        self.converged = None
        self.phi = None
        self.functional = None
        self.result = None

    def _total(self):
        ev = self.EnergyEvaluator
        if isinstance(ev, TotalFunctional):
            if not ev._fusable():
                raise NotImplementedError("the energy evaluator's functionals cannot be fused on the device")
            return ev
        if isinstance(ev, NativeFunctional):
            return TotalFunctional(F=ev)
        raise NotImplementedError("the energy evaluator must be built from dftpy_gb300 functionals")

    def options_struct(self):
        o = self.optimization_options
        s = _lib.OptOptions()
        _lib.load().ofdft_opt_default(_lib.C.byref(s))
        if self._method_code is None:
            raise AttributeError("The %s direction method not implemented." % self.optimization_method)
        s.method = self._method_code
        s.maxiter, s.maxfun, s.maxls = int(o["maxiter"]), int(o["maxfun"]), int(o["maxls"])
        s.ncheck, s.maxcor = int(o["ncheck"]), int(o["maxcor"])
        s.econv = float(o["econv"]) if o["econv"] is not None else 0.0
        s.c1, s.c2, s.xtol = float(o["c1"]), float(o["c2"]), float(o["xtol"])
        s.h0 = float(o["h0"]) if o["h0"] else 0.0
        s.verbose = 1 if self.verbose else 0
        # not in the reference: a residual stop and a derivative-only line search
        # (for float32 stages whose energies are noisier than the last decreases)
        s.pconv = float(o["pconv"]) if o["pconv"] else 0.0
        if o["linesearch"] not in ("wolfe", "grad"):
            raise ValueError("linesearch must be 'wolfe' (the reference's) or 'grad'")
        s.ls_grad = 1 if o["linesearch"] == "grad" else 0
        # not in the reference either: L-BFGS and TN may start each line search at the
        # direction's own length (the quasi-Newton step) instead of theta = 1
        if o["linesearch_start"] not in ("reference", "direction"):
            raise ValueError("linesearch_start must be 'reference' or 'direction'")
        s.ls_start = 1 if o["linesearch_start"] == "direction" else 0
        return s

    def optimize_rho(self, guess_rho=None, guess_phi=None, lphi=False, lsfun="line_search", dtype=None):
        if guess_rho is None and self.rho is None:
            raise AttributeError("Must provide a guess density")
        if guess_rho is not None:
            self.rho = guess_rho
        if guess_phi is not None:
            raise NotImplementedError("guess_phi is not supported")
        total = self._total()
        rho0 = self.rho
        grid = rho0.grid if isinstance(rho0, DirectField) else next(
            f.grid for f in total.funcDict.values() if getattr(f, "grid", None) is not None)
        rho = DirectField(grid, data=rho0, dtype=dtype or (rho0.dtype if isinstance(rho0, torch.Tensor)
                                                           else torch.float64)).clone()
        ev = total.evaluator(grid, rho.dtype)
        total.prepare(ev, grid, rho.dtype)
        res = _lib.OptResult()
        opts = self.options_struct()
        t = rho.as_subclass(torch.Tensor)
        V = torch.empty_like(t)
        _lib.check(_lib.load().ofdft_optimize_v(ev.h, _lib.C.c_void_p(t.data_ptr()), _lib.C.byref(opts),
                                                _lib.C.byref(res), _lib.C.c_void_p(V.data_ptr()), stream_ptr()))
        total.finish(ev)
        rho._N = None
        self.result = res
        self.converged = res.converged
        self.mu = res.mu
        self.rho = rho
        self.phi = torch.sqrt(rho)
        # the last accepted evaluation (optimization.py:517-523): no further evaluation
        v = V.as_subclass(DirectField)
        v.grid = grid
        v._N = None
        self.functional = FunctionalOutput(name="TOTAL", energy=float(res.energy), potential=v)
        return rho

    def optimize_rho_mixed(self, guess_rho=None, econv_f32=None, f32_method=None, refine_method=None,
                           refine_maxiter=None, refine="optimize", f32_options=None, f32_polish=None):
        """FP32-mixed ground state with a final FP64 refinement.

        Stage 1 optimises in FP32-mixed (float32 fields and FFTs, float64
        reductions) until the energy changes by less than ``econv_f32``
        (default 10x the FP64 econv) or the line search can make no progress.
        Stage 2, ``refine="optimize"``: continues in FP64 from that density with
        the FP64 econv, so the converged energy and density are those of the
        FP64 functional.  ``refine="evaluate"``: one FP64 E+V evaluation of the
        stage-1 density (electron count restored in float64), whose energy and
        potential become the result.
        ``f32_options``: options of the FP32 stage over these.
        ``f32_polish``: a dict of options (e.g. ``{"pconv": 2e-6, "maxiter": 150}``)
        for a second FP32 L-BFGS stage from the first one's density on the
        derivative-only line search (``linesearch="grad"``, no energy test): it
        converges on the float32 gradient, which stays accurate where float32
        energies no longer resolve the decreases, so the FP64 refinement starts
        at the FP32 functional's own stationary point.
        Returns the FP64 density; ``self.stages`` records both stages."""
        if refine not in ("optimize", "evaluate"):
            raise ValueError("refine must be 'optimize' or 'evaluate'")
        if guess_rho is not None:
            self.rho = guess_rho
        o = dict(self.optimization_options)
        econv64 = o["econv"]
        stages = []
        m32 = f32_method or ("LBFGS" if self.optimization_method == "TN" else self.optimization_method)
        o32 = dict(o, econv=econv_f32 if econv_f32 is not None else 10.0 * econv64)
        o32.update(f32_options or {})
        opt32 = Optimization(m32, o32, self.EnergyEvaluator)
        opt32.verbose = self.verbose
        rho32 = opt32.optimize_rho(guess_rho=self.rho, dtype=torch.float32)
        stages.append({"precision": "f32", "method": m32, "niter": opt32.result.niter,
                       "nfev": opt32.result.nfev, "converged": opt32.converged, "energy": opt32.result.energy,
                       "dP": opt32.result.dP})
        if f32_polish is not None:
            op = dict(o32, econv=0.0, linesearch="grad", maxiter=150)
            op.update(f32_polish)
            optp = Optimization("LBFGS", op, self.EnergyEvaluator)
            optp.verbose = self.verbose
            rho32 = optp.optimize_rho(guess_rho=rho32, dtype=torch.float32)
            stages.append({"precision": "f32", "method": "LBFGS, derivative line search",
                           "niter": optp.result.niter, "nfev": optp.result.nfev, "converged": optp.converged,
                           "energy": optp.result.energy, "dP": optp.result.dP})
            opt32 = optp
        o64 = dict(o)
        if refine_maxiter is not None:
            o64["maxiter"] = refine_maxiter
        opt64 = Optimization(refine_method or self.optimization_method, o64, self.EnergyEvaluator)
        opt64.verbose = self.verbose
        # float32 fields keep the electron count only to ~1e-7; the FP64 stage
        # conserves whatever count it starts from, so restore the guess's count
        guess = self.rho if isinstance(self.rho, DirectField) else DirectField(rho32.grid, data=self.rho)
        n_target = DirectField(rho32.grid, data=guess, dtype=torch.float64).integral()
        rho_start = rho32.as_subclass(torch.Tensor).double()
        n32 = DirectField(rho32.grid, data=rho_start).integral()
        if refine == "evaluate":
            rho = DirectField(rho32.grid, data=rho_start * (n_target / n32))
            total = self._total()
            func = total(rho, calcType={"E", "V"})
            res = opt32.result
            stages.append({"precision": "f64", "method": "evaluate", "niter": 0, "nfev": 1,
                           "converged": opt32.converged, "energy": func.energy})
            self.stages = stages
            self.result = res
            self.converged = opt32.converged
            self.mu = float((func.potential * rho).integral() / rho.integral())
            self.rho = rho
            self.phi = torch.sqrt(rho)
            self.functional = func
            return rho
        rho = opt64.optimize_rho(guess_rho=rho_start * (n_target / n32), dtype=torch.float64)
        stages.append({"precision": "f64", "method": opt64.optimization_method, "niter": opt64.result.niter,
                       "nfev": opt64.result.nfev, "converged": opt64.converged, "energy": opt64.result.energy})
        self.stages = stages
        self.result = opt64.result
        self.converged = opt64.converged
        self.mu = opt64.mu
        self.rho = rho
        self.phi = opt64.phi
        self.functional = opt64.functional
        return rho

    def __call__(self, guess_rho=None, calcType={"E", "V"}, guess_phi=None, lphi=False):
        return self.optimize_rho(guess_rho=guess_rho, guess_phi=guess_phi, lphi=lphi)


_BATCH_MAX = 128


def optimize_rho_batch(optimizations, guess_rhos, dtype=None, refine=None, persistent=False):
    """Ground states of many independent systems together.

    ``optimizations`` are ``Optimization`` objects (L-BFGS, one per system, each
    with its own energy evaluator and grid; options equal except ``econv``).
    All systems run the L-BFGS of ``optimize_rho`` in lockstep on the device
    (``ofdft_optimize_batch``): every vector operation is one launch for the
    whole batch and every round of scalars one synchronisation, instead of one
    per system.  Each system's result is the one ``optimize_rho`` gives it.

    ``dtype``: field precision of the optimisation (default float64).
    ``refine="evaluate"``: after a float32 optimisation, evaluate every density
    once in FP64 (electron count restored in float64), as
    ``optimize_rho_mixed(refine="evaluate")`` does for one system.
    ``persistent=True``: every round of evaluations runs as one persistent
    cooperative launch for all active systems (``dftpy_gb300.batch``, launch
    shape from the autotuner), replayed as a CUDA graph, when every system's
    functional is eligible (TF, vW, LDA, Hartree, local PP); the results then
    equal the single solves to rounding, not bit for bit.
    Returns the densities; each ``Optimization`` gets ``rho``, ``mu``,
    ``converged``, ``result`` and ``functional``."""
    opts = list(optimizations)
    guesses = list(guess_rhos)
    if len(opts) != len(guesses):
        raise ValueError("one guess density per optimisation")
    if not opts:
        return []
    dtype = dtype or torch.float64
    base = opts[0].options_struct()
    for o in opts:
        if o.optimization_method != "LBFGS":
            raise NotImplementedError("optimize_rho_batch runs L-BFGS only")
        s = o.options_struct()
        for f, _ in _lib.OptOptions._fields_:
            if f != "econv" and getattr(s, f) != getattr(base, f):
                raise ValueError("batched optimisations must share every option but econv (%s differs)" % f)
    base.batch_persistent = 1 if persistent else 0
    lib = _lib.load()
    out = []
    for c0 in range(0, len(opts), _BATCH_MAX):
        chunk = list(zip(opts[c0:c0 + _BATCH_MAX], guesses[c0:c0 + _BATCH_MAX]))
        n = len(chunk)
        totals, evs, rhos, vs, grids = [], [], [], [], []
        for o, guess in chunk:
            total = o._total()
            grid = guess.grid if isinstance(guess, DirectField) else next(
                f.grid for f in total.funcDict.values() if getattr(f, "grid", None) is not None)
            rho = DirectField(grid, data=guess, dtype=dtype).clone()
            ev = total.evaluator(grid, rho.dtype)
            total.prepare(ev, grid, rho.dtype)
            totals.append((total, ev))
            evs.append(ev.h)
            rhos.append(rho)
            vs.append(torch.empty_like(rho.as_subclass(torch.Tensor)))
            grids.append(grid)
        P = _lib.C.c_void_p
        ev_arr = (P * n)(*[P(h.value if hasattr(h, "value") else h) for h in evs])
        rho_arr = (P * n)(*[P(r.as_subclass(torch.Tensor).data_ptr()) for r in rhos])
        v_arr = (P * n)(*[P(v.data_ptr()) for v in vs])
        econv = (_lib.C.c_double * n)(*[float(o.optimization_options["econv"] or 0.0) for o, _ in chunk])
        res = (_lib.OptResult * n)()
        _lib.check(lib.ofdft_optimize_batch(n, ev_arr, rho_arr, _lib.C.byref(base), econv, res, v_arr, stream_ptr()))
        for i, (o, _) in enumerate(chunk):
            total, ev = totals[i]
            total.finish(ev)
            rho = rhos[i]
            rho._N = None
            r = res[i]
            o.result = r
            o.converged = r.converged
            o.mu = r.mu
            v = vs[i].as_subclass(DirectField)
            v.grid = grids[i]
            v._N = None
            o.functional = FunctionalOutput(name="TOTAL", energy=float(r.energy), potential=v)
            if refine == "evaluate" and rho.dtype != torch.float64:
                n_target = DirectField(grids[i], data=chunk[i][1], dtype=torch.float64).integral()
                r64 = DirectField(grids[i], data=rho.as_subclass(torch.Tensor).double())
                r64 = DirectField(grids[i], data=r64 * (n_target / r64.integral()))
                func = total(r64, calcType={"E", "V"})
                o.stages = [{"precision": "f32", "method": "LBFGS", "niter": r.niter, "nfev": r.nfev,
                             "converged": r.converged, "energy": r.energy},
                            {"precision": "f64", "method": "evaluate", "niter": 0, "nfev": 1,
                             "converged": r.converged, "energy": func.energy}]
                o.functional = func
                o.mu = float((func.potential * r64).integral() / r64.integral())
                rho = r64
            o.rho = rho
            o.phi = torch.sqrt(rho)
            out.append(rho)
    return out


class OESCF:
    """OE-SCF (src/dftpy/optimization/scf.py:6-119): the nonlocal part of the
    kinetic functional (``evaluator_emb``) is frozen as an external potential,
    the density is optimised with the rest (``optimization``, vW and the other
    terms) on the device, and the outer loop mixes the densities (``mixer``,
    dftpy_gb300.mixer) until the energy changes by less than econv.  The inner
    convergence threshold tightens with the Hartree energy of the density
    change (scf.py:62-81)."""

    def __init__(self, optimization=None, evaluator_emb=None, guess_rho=None, mixer=None, maxiter=0):
        from .functional.external_potential import ExternalPotential
        self.optimization = optimization
        self.evaluator_emb = evaluator_emb
        self.rho = guess_rho
        self.mixer = mixer
        self.maxiter = maxiter
        self.iter = 0
        self.residual_norm_prev = 1.0
        if self.maxiter < 1:
            self.maxiter = self.options["maxiter"]
        self.extfunctional = ExternalPotential()
        self.error = 1.0
        self.converged = False

    @property
    def options(self):
        return self.optimization.optimization_options

    def optimize_rho(self, **kwargs):
        return self.run(**kwargs)

    def run(self, guess_rho=None, **kwargs):
        if guess_rho is None and self.rho is None:
            raise AttributeError("Must provide a guess density")
        elif guess_rho is not None:
            self.rho = guess_rho
        self.ncharges = float(self.rho.integral())
        self.econv = self.options["econv"] * 1.0
        self.energyhistory = []
        self.inner_stats = []  # per outer iteration: inner iterations, evaluations, econv
        self.converged = False
        for i in range(self.maxiter):
            self.get_density()
            self.mix()
            if self.error < self.econv:
                self.converged = True
                break
        return self.rho

    def get_density(self, norm=None, **kwargs):
        self.iter += 1
        scale = 1e-2
        if norm is None:
            if self.iter == 1:
                norm = self.ncharges * 1e-1
                self.options["econv"] = 1e10
            elif self.iter == 2:
                norm = self.ncharges * 1e-3
            else:
                norm = self.dp_norm
        econv = max(norm * scale, 1e-7 * self.ncharges)
        if econv < self.options["econv"]:
            self.options["econv"] = econv
        self.iterative(**kwargs)

    def iterative(self, **kwargs):
        self.rho_prev = self.rho.clone()
        func = self.evaluator_emb(self.rho, calcType={"E", "V"})
        self.extfunctional.v = func.potential
        self.extenergy = func.energy - self.extfunctional(self.rho, calcType={"E"}).energy
        funcs = self.optimization.EnergyEvaluator.funcDict
        funcs["EMB"] = self.extfunctional
        try:
            self.optimization.optimize_rho(guess_rho=self.rho)
        finally:
            del funcs["EMB"]
        self.rho = self.optimization.rho
        res = self.optimization.result
        if res is not None:
            self.inner_stats.append({"niter": res.niter, "nfev": res.nfev, "econv": self.options["econv"]})
        self.functional = self.optimization.functional
        self.functional.energy += self.extenergy
        energy = self.functional.energy
        if len(self.energyhistory) > 0:
            self.error = abs(energy - self.energyhistory[-1])
        else:
            self.error = abs(energy)
        self.energyhistory.append(energy)

    def mix(self, **kwargs):
        from .functional.semilocal import Hartree
        r = self.rho - self.rho_prev
        self.dp_norm = Hartree.compute(r, calcType={"E"}).energy
        if self.iter == 1:
            self.dp_norm_prev = self.dp_norm
        else:
            self.dp_norm, self.dp_norm_prev = self.dp_norm_prev, self.dp_norm
            self.dp_norm = (self.dp_norm + self.dp_norm_prev) / 2
        if self.mixer:
            self.rho = self.mixer(self.rho_prev, self.rho, **kwargs)
