"""The FP32-mixed ground state with the float32 polish stage (FP32 L-BFGS, then
FP32 L-BFGS on the derivative-only line search, then one FP64 E+V) against a
tightly converged FP64 ground state: energy within 1e-6 Ha/atom and PP + Ewald
forces within 1e-5 Ha/Bohr (the benchmark spec's bars), and the polish stage lowers the
float32 residual below the energy line search's stall.  32 displaced Al atoms
on 48^3, WT + LDA + Hartree + PME local PP; and the headline's k_F-node kernel
(Hermite interpolation, fixed k_F bounds, 16 nodes) on 4 atoms at 32^3; with
the reference's first trial step (theta = 1) and with the direction's own
length (the quasi-Newton step) as the first trial step of every line search.
The direction start also reaches the FP64 ground state of the reference start
in fewer evaluations."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn

WGC = dict(alpha=(5 + 5 ** 0.5) / 6, beta=(5 - 5 ** 0.5) / 6)


def _system(reps, n, kedf):
    lat, pos = syn.fcc_supercell(7.6, reps, sigma=0.1, seed=7)
    nat = len(pos)
    gp, vp = syn.analytic_vloc(3.0, 1.0)
    grid = D.DirectGrid(lat, (n, n, n))
    ions = D.Ions(symbols=["Al"] * nat, positions=pos, cell=lat)
    pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": D.functional.RECPOT(r=gp, v=vp, zval=3)}, PME=True)
    tot = D.TotalFunctional(KineticEnergyFunctional=kedf, XCFunctional=D.Functional(type="XC", name="LDA"),
                            HARTREE=D.Functional(type="HARTREE"), PSEUDO=pp)
    return nat, grid, tot, D.DirectField(grid) + 3.0 * nat / grid.volume


@pytest.mark.parametrize("start", ["reference", "direction"])
@pytest.mark.parametrize("case", ["wt", "lwt_hermite"])
def test_mixed_polish_meets_the_ground_state_bars(case, start):
    torch.cuda.set_device(0)
    if case == "wt":
        nat, grid, tot, rho0 = _system(2, 48, D.Functional(type="KEDF", name="WT"))
    else:
        ke = D.Functional(type="KEDF", name="LWT", nsp=16, kdd=3, interp="hermite", kfmin=0.3, kfmax=3.0, **WGC)
        nat, grid, tot, rho0 = _system(1, 32, ke)
    ref = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS",
                         optimization_options={"econv": 1e-12 * nat, "maxiter": 800, "maxfun": 50})
    r_ref = ref.optimize_rho(guess_rho=rho0)
    f_ref = tot.get_forces(r_ref)
    o = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS",
                       optimization_options={"econv": 1e-10 * nat, "maxiter": 800, "maxfun": 50})
    rm = o.optimize_rho_mixed(guess_rho=rho0, econv_f32=1e-9 * nat, refine="evaluate",
                              f32_options={"linesearch_start": start},
                              f32_polish={"maxiter": 150, "linesearch_start": start})
    assert rm.dtype == torch.float64
    assert len(o.stages) == 3 and o.stages[1]["method"].startswith("LBFGS, derivative")
    assert o.stages[1]["dP"] < o.stages[0]["dP"]
    assert abs(o.functional.energy - ref.functional.energy) / nat <= 1e-6
    assert float(np.abs(tot.get_forces(rm) - f_ref).max()) <= 1e-5
    assert abs(float(rm.integral()) - float(rho0.integral())) <= 1e-10 * float(rho0.integral())


def test_direction_start_same_ground_state_fewer_evaluations():
    torch.cuda.set_device(0)
    nat, grid, tot, rho0 = _system(2, 48, D.Functional(type="KEDF", name="WT"))
    runs = {}
    for start in ("reference", "direction"):
        o = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS",
                           optimization_options={"econv": 1e-11 * nat, "maxiter": 800, "maxfun": 50,
                                                 "linesearch_start": start})
        r = o.optimize_rho(guess_rho=rho0)
        runs[start] = (o.functional.energy, tot.get_forces(r), o.result.nfev, o.converged)
    (e_r, f_r, n_r, c_r), (e_d, f_d, n_d, c_d) = runs["reference"], runs["direction"]
    assert c_r == 0 and c_d == 0
    assert abs(e_d - e_r) / nat <= 1e-8
    assert float(np.abs(f_d - f_r).max()) <= 1e-5
    assert n_d < n_r, (n_d, n_r)
