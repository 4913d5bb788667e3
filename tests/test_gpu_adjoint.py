"""Adjoint gradients on the device: dE/drho, dE/dR and dE/d(radial PP table),
each against central finite differences, the table gradient also against the
oracle's energy, and the FP32-mixed adjoint against the FP64 one."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn
from dftpy_gb300.autograd import energy_and_gradients, total_energy
from oracle import ofdft_np as O


def _system(pme=True, nr=(24, 20, 18), two=True):
    lat, pos = syn.fcc_cell(7.6)
    pos = pos + np.random.default_rng(4).normal(0, 0.15, pos.shape)
    sym = ["Al", "Mg", "Al", "Mg"] if two else ["Al"] * 4
    ga, va = syn.analytic_vloc(3.0, 1.0, npts=256)
    gb, vb = syn.analytic_vloc(2.0, 1.2, npts=256)
    tabs = {"Al": D.functional.RECPOT(r=ga, v=va, zval=3), "Mg": D.functional.RECPOT(r=gb, v=vb, zval=2)}
    if not two:
        tabs.pop("Mg")
    grid = D.DirectGrid(lat, nr)
    ions = D.Ions(symbols=sym, positions=pos, cell=lat)
    pp = D.LocalPseudo(grid=grid, ions=ions, PP_list=tabs, PME=pme)
    tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="WT"),
                            XCFunctional=D.Functional(type="XC", name="LDA"), HARTREE=D.Functional(type="HARTREE"),
                            PSEUDO=pp)
    nel = sum(3.0 if s == "Al" else 2.0 for s in sym)
    rho = syn.smooth_density(lat, nr, nel, seed=8, amp=0.3)
    return lat, pos, sym, tabs, grid, pp, tot, rho


@pytest.mark.parametrize("pme", [True, False])
def test_table_gradient_vs_oracle_fd(pme):
    lat, pos, sym, tabs, grid, pp, tot, rho = _system(pme)
    g = pp.vloc_grad(D.DirectField(grid, data=rho))
    og = O.Grid(lat, grid.nrR)
    keys = sorted(tabs)
    spec = np.array([keys.index(s) for s in sym])
    base = [(tabs[k].r, tabs[k].v.copy()) for k in keys]

    def e_pp(tables):
        return O.LocalPseudo(og, pos, spec, tables, PME=pme)(rho, ("E",))["E"]

    scale = max(np.abs(g[k]).max() for k in keys)
    for si, k in enumerate(keys):
        for idx in (0, 1, 2, 3, 7, 40, 200, 254):
            h = 1e-3 * max(1.0, abs(base[si][1][idx]))
            tp = [(r, v.copy()) for r, v in base]
            tm = [(r, v.copy()) for r, v in base]
            tp[si][1][idx] += h
            tm[si][1][idx] -= h
            fd = (e_pp(tp) - e_pp(tm)) / (2 * h)
            assert abs(fd - g[k][idx]) <= 1e-8 * max(1.0, scale), (k, idx, fd, g[k][idx])


def test_autograd_rho_positions_tables():
    lat, pos, sym, tabs, grid, pp, tot, rho_np = _system(True)
    rho = torch.tensor(rho_np, device="cuda", requires_grad=True)
    R = torch.tensor(pos, dtype=torch.float64, requires_grad=True)
    keys = pp.species_keys
    T = torch.tensor(np.concatenate([tabs[k].v for k in keys]), requires_grad=True)
    E = total_energy(tot, rho, R, T)
    E.backward()
    # dE/drho: directional derivative
    d = torch.tensor(syn.smooth_density(lat, grid.nrR, 1.0, seed=3, amp=0.5) - 1.0 / grid.volume, device="cuda")
    h = 1e-4
    ep = float(total_energy(tot, (rho + h * d).detach(), R.detach(), T.detach()))
    em = float(total_energy(tot, (rho - h * d).detach(), R.detach(), T.detach()))
    fd = (ep - em) / (2 * h)
    an = float((rho.grad * d).sum())
    assert abs(fd - an) < 1e-7 * max(1.0, abs(an)), (fd, an)
    # dE/dR: central differences of E (PP + Ewald move with the atoms), h = 1e-4 Bohr
    for a, c in ((0, 0), (1, 2), (3, 1)):
        Rp = R.detach().clone()
        Rm = R.detach().clone()
        Rp[a, c] += 1e-4
        Rm[a, c] -= 1e-4
        ep = float(total_energy(tot, rho.detach(), Rp, T.detach()))
        em = float(total_energy(tot, rho.detach(), Rm, T.detach()))
        fd = (ep - em) / 2e-4
        assert abs(fd - float(R.grad[a, c])) < 1e-6, (a, c, fd, float(R.grad[a, c]))
    # dE/dtables: E is linear in the table, central difference is exact up to rounding
    for idx in (0, 5, 120, 256 + 3, 256 + 90):
        Tp = T.detach().clone()
        Tm = T.detach().clone()
        h = 1e-3
        Tp[idx] += h
        Tm[idx] -= h
        ep = float(total_energy(tot, rho.detach(), R.detach(), Tp))
        em = float(total_energy(tot, rho.detach(), R.detach(), Tm))
        fd = (ep - em) / (2 * h)
        assert abs(fd - float(T.grad[idx])) < 1e-8 * max(1.0, float(T.grad.abs().max())), (idx, fd,
                                                                                            float(T.grad[idx]))


def test_fp32_adjoint_vs_fp64():
    lat, pos, sym, tabs, grid, pp, tot, rho_np = _system(True)
    E64, V64, dR64, dT64 = energy_and_gradients(tot, D.DirectField(grid, data=rho_np))
    E32, V32, dR32, dT32 = energy_and_gradients(tot, D.DirectField(grid, data=rho_np, dtype=torch.float32))
    assert abs(E32 - E64) / 4 < 1e-5
    assert np.abs(dR32 - dR64).max() < 1e-4
    assert np.abs(dT32 - dT64).max() < 1e-5 * max(1.0, np.abs(dT64).max())


def test_mixed_ground_state_matches_fp64(golden):
    """FP32-mixed optimisation + FP64 refinement reaches the FP64 ground state."""
    from dftpy_gb300 import synthetic as syn2
    lat, pos = syn2.fcc_cell(7.60)
    grid = D.DirectGrid(lat, (32, 32, 32))
    ions = D.Ions(symbols=["Al"] * 4, positions=pos, cell=lat)
    rp = D.functional.RECPOT(r=golden["recpot_gp"], v=golden["recpot_vp"], zval=3)
    pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": rp}, PME=True)
    tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="TFVW"),
                            XCFunctional=D.Functional(type="XC", name="LDA"), HARTREE=D.Functional(type="HARTREE"),
                            PSEUDO=pp)
    rho0 = D.DirectField(grid) + 12.0 / grid.volume
    opt = D.Optimization(EnergyEvaluator=tot, optimization_method="TN",
                         optimization_options={"econv": 1e-11 * 4, "maxiter": 80, "maxfun": 50})
    rho = opt.optimize_rho_mixed(guess_rho=rho0, econv_f32=1e-6)
    assert opt.converged == 0
    assert rho.dtype == torch.float64
    ref = float(golden["C_TN_E"])
    assert abs(tot.Energy(rho) - ref) <= 1e-10 * abs(ref)
    assert opt.stages[0]["precision"] == "f32" and opt.stages[1]["precision"] == "f64"
