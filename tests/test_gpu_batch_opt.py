"""GPU checks of the lockstep batched L-BFGS (ofdft_optimize_batch): every
system of a batch of uneven grids gets exactly the result of solving it on its
own with Optimization.optimize_rho (same energy, iteration count and density,
bit for bit), in FP64 and FP32, with per-system econv."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn
from dftpy_gb300.optimization import optimize_rho_batch

SHAPES = [("fcc", 1, (24, 24, 24), 7.6), ("bcc", 2, (32, 32, 32), 7.4), ("sc", 2, (20, 24, 28), 7.8),
          ("fcc", 1, (30, 30, 30), 7.3), ("sc", 3, (36, 36, 36), 7.5)]


def _systems(dtype):
    gp, vp = syn.analytic_vloc(3.0, 1.0)
    cells = {"fcc": syn.fcc_cell, "bcc": syn.bcc_cell, "sc": syn.sc_cell}
    out = []
    rng = np.random.default_rng(11)
    for kind, reps, nr, a in SHAPES:
        lat, pos = cells[kind](a)
        lat, pos = syn.supercell(lat, pos, (reps, reps, reps))
        pos = pos + rng.normal(0.0, 0.1, size=pos.shape)
        nat = len(pos)
        grid = D.DirectGrid(lat, nr)
        ions = D.Ions(symbols=["Al"] * nat, positions=pos, cell=lat)
        pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": D.functional.RECPOT(r=gp, v=vp, zval=3)}, PME=True)
        tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="TFVW"),
                                XCFunctional=D.Functional(type="XC", name="LDA"),
                                HARTREE=D.Functional(type="HARTREE"), PSEUDO=pp)
        rho0 = D.DirectField(grid, dtype=dtype) + 3.0 * nat / grid.volume
        out.append((tot, rho0, nat))
    return out


def _opt(tot, nat, econv_pa, start="reference"):
    return D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS",
                          optimization_options={"econv": econv_pa * nat, "maxiter": 200, "maxfun": 50,
                                                "linesearch_start": start})


@pytest.mark.parametrize("start", ["reference", "direction"])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batch_equals_single_solves(dtype, start):
    """Also with every line search started at the scaled length of the L-BFGS
    direction (linesearch_start="direction"), whose lengths the batch computes
    on the device."""
    systems = _systems(dtype)
    econvs = [1e-7, 1e-8, 1e-7, 1e-6, 1e-7]
    singles = []
    for (tot, rho0, nat), ec in zip(systems, econvs):
        o = _opt(tot, nat, ec, start)
        r = o.optimize_rho(guess_rho=rho0, dtype=dtype)
        singles.append((o, r))
    batch = [_opt(tot, nat, ec, start) for (tot, rho0, nat), ec in zip(systems, econvs)]
    rhos = optimize_rho_batch(batch, [rho0 for _, rho0, _ in systems], dtype=dtype)
    for (o1, r1), o2, r2 in zip(singles, batch, rhos):
        assert o2.converged == o1.converged
        assert o2.result.niter == o1.result.niter and o2.result.nfev == o1.result.nfev
        assert o2.functional.energy == o1.functional.energy
        assert o2.mu == o1.mu
        assert torch.equal(r2.as_subclass(torch.Tensor), r1.as_subclass(torch.Tensor))
        assert torch.equal(o2.functional.potential.as_subclass(torch.Tensor),
                           o1.functional.potential.as_subclass(torch.Tensor))


def test_batch_mixed_refinement_matches_fp64():
    """FP32 batch + one FP64 evaluation per system: within the FP32-mixed bar of
    the FP64 ground state (|dE| <= 1e-6 Ha/atom)."""
    sys64 = _systems(torch.float64)
    e64 = []
    for tot, rho0, nat in sys64:
        o = _opt(tot, nat, 1e-7)
        o.optimize_rho(guess_rho=rho0)
        e64.append(o.functional.energy)
    batch = [_opt(tot, nat, 1e-7) for tot, _, nat in sys64]
    optimize_rho_batch(batch, [rho0 for _, rho0, _ in sys64], dtype=torch.float32, refine="evaluate")
    for o, e, (_, _, nat) in zip(batch, e64, sys64):
        assert o.converged == 0
        assert abs(o.functional.energy - e) / nat <= 1e-6


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_persistent_batch_matches_single_solves(dtype):
    """persistent=True: every round of evaluations in one cooperative launch
    (replayed as a graph).  Its transforms are the library's own, not cuFFT,
    so a system's path can move by an iteration where an energy difference
    sits at the econv threshold: every system converges, its energy within
    its econv per atom (1e-7 Ha/atom) of the single solve, FP64; FP32 within
    1e-6 Ha/atom."""
    global SHAPES
    saved = SHAPES
    SHAPES = [s if s[2] != (20, 24, 28) else (s[0], s[1], (20, 24, 30), s[3]) for s in saved]
    try:
        systems = _systems(dtype)
    finally:
        SHAPES = saved
    singles = []
    for tot, rho0, nat in systems:
        o = _opt(tot, nat, 1e-7)
        o.optimize_rho(guess_rho=rho0, dtype=dtype)
        singles.append(o)
    batch = [_opt(tot, nat, 1e-7) for tot, _, nat in systems]
    optimize_rho_batch(batch, [rho0 for _, rho0, _ in systems], dtype=dtype, persistent=True)
    bar = 1e-7 if dtype == torch.float64 else 1e-6
    for o1, o2, (_, _, nat) in zip(singles, batch, systems):
        assert o2.converged == 0 and o1.converged == 0
        assert abs(o2.functional.energy - o1.functional.energy) / nat <= bar, (o2.functional.energy,
                                                                              o1.functional.energy)
