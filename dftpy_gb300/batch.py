"""Many independent systems of uneven size on one GPU.

``optimize_many`` runs one density optimisation per system concurrently: a
pool of host threads, each driving the native optimiser of its system on its
own CUDA stream.  ctypes releases the GIL for the whole native call, so the
systems' kernels and transforms interleave on the GPU and small grids (which
alone leave most of the 152 SMs idle) fill the device together.  Every system
keeps its own grid handle, evaluator, plans and scratch, so no state is
shared between streams.
"""
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import torch

from .optimization import Optimization

__all__ = ["optimize_many"]


def optimize_many(totals, guesses, method="LBFGS", options=None, mixed=False, threads=16, econv_f32=None):
    """Optimise every (total functional, guess density) pair.

    mixed=False runs each system in the precision of its guess; mixed=True runs
    FP32-mixed followed by an FP64 refinement (Optimization.optimize_rho_mixed).
    Returns a list of dicts (energy, converged, niter, nfev, seconds, rho) in
    input order, plus the wall time of the whole batch."""
    results = [None] * len(totals)
    device = torch.cuda.current_device()

    def run(i):
        torch.cuda.set_device(device)
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            opt = Optimization(method, dict(options or {}), totals[i])
            t0 = time.perf_counter()
            if mixed:
                rho = opt.optimize_rho_mixed(guess_rho=guesses[i], econv_f32=econv_f32)
            else:
                rho = opt.optimize_rho(guess_rho=guesses[i])
            stream.synchronize()
            results[i] = {"energy": float(opt.functional.energy), "converged": int(opt.converged),
                          "niter": int(opt.result.niter), "nfev": int(opt.result.nfev),
                          "seconds": time.perf_counter() - t0, "rho": rho,
                          "stages": getattr(opt, "stages", None)}

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        list(ex.map(run, range(len(totals))))
    torch.cuda.synchronize()
    return results, time.perf_counter() - t0
