"""GPU parity of the GGA kinetic functionals (kedf/gga.py) against the
reference's outputs (tests/golden/make_golden_gga.py): every functional of the
reference's list, energy, potential and stress in FP64; the reference's own
'lc94' test; FP32-mixed against FP64; and a ground state with a GGA kinetic
term.

Bars: FP64 energy within 1e-10 relative, potential within 1e-9 of max|V|,
stress within 1e-9 of its largest component; FP32 energy within 2e-6
relative, potential within 1e-4 of max|V| (float32 gradients divided by
rho^(4/3))."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn

HERE = os.path.dirname(os.path.abspath(__file__))
GG = dict(np.load(os.path.join(HERE, "golden", "reference_gga.npz")))
CASES = [(str(n), str(n), {}) for n in GG["names"]] + [("LKT_P", "LKT", {"params": [1.1, 0.9]}),
                                                       ("LKT_RVW", "LKT", {"gga_remove_vw": 1.0}),
                                                       ("LKT_SIG", "LKT", {"sigma": 0.2}), ("LC94_SIG", "LC94", {"sigma": 0.35})]


def _np(f):
    return f.as_subclass(torch.Tensor).double().cpu().numpy()


@pytest.mark.parametrize("tag,name,kw", CASES, ids=[c[0] for c in CASES])
def test_gga_fp64_against_reference(golden, tag, name, kw):
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    f = D.Functional(type="KEDF", name="GGA", k_str=name, **kw)
    o = f(rho)
    e = GG["A_E_" + tag]
    assert abs(o.energy - e) <= 1e-10 * max(1.0, abs(e)), (o.energy, e)
    v = GG["A_V_" + tag]
    assert float(np.abs(_np(o.potential) - v).max()) <= 1e-9
    s = GG["A_S_" + tag]
    st = f.stress(rho)
    assert float(np.abs(st - s).max()) <= 1e-9 * max(1e-12, float(np.abs(s).max()))


def test_gga_reference_fixture(golden):
    """The reference's own test (test_functional.py:10-21): GGA 'lc94' on Al_fde_rho.pp."""
    grid = D.DirectGrid(golden["E_lattice"], golden["E_nr"])
    rho = D.DirectField(grid, data=golden["E_rho"])
    func = D.Functional(type="KEDF", name="GGA", k_str="lc94")(rho)
    assert abs(func.energy - GG["fixture_E_LC94"]) <= 1e-10 * abs(func.energy)
    assert np.isclose(func.energy, 1.6821337114254904)
    assert np.isclose((func + func).energy, 1.6821337114254904 * 2)
    assert np.isclose((func * 2).energy, 1.6821337114254904 * 2)
    assert np.isclose((func / 2).energy, 1.6821337114254904 / 2)


@pytest.mark.parametrize("name", ["LKT", "LC94", "REVAPBEK", "PBE4"])
def test_gga_fp32_against_fp64(name):
    nr = (64, 64, 64)
    lat = np.diag([15.2, 15.2, 15.2])
    rho_np = syn.smooth_density(lat, nr, 32.0, seed=12, amp=0.5)
    grid = D.DirectGrid(lat, nr)
    out = {}
    for dt in (torch.float64, torch.float32):
        o = D.Functional(type="KEDF", name="GGA", k_str=name)(D.DirectField(grid, data=rho_np, dtype=dt))
        out[dt] = (o.energy, _np(o.potential))
    (e64, v64), (e32, v32) = out[torch.float64], out[torch.float32]
    assert abs(e32 - e64) <= 2e-6 * abs(e64), (e32, e64)
    assert float(np.abs(v32 - v64).max()) <= 1e-4 * float(np.abs(v64).max())


def test_gga_ground_state():
    """L-BFGS with GGA (LKT) + LDA + Hartree + PME PP converges in FP64, and the
    mixed solver (FP32 stage, FP64 L-BFGS continuation) reaches the same energy.
    The FP32 stage alone can stop at its first line search: trial rotations of
    phi reach near-zero densities, where the GGA potential is large and float32
    gradients of rho carry relative errors of order one."""
    lat, pos = syn.fcc_cell(7.6)
    gp, vp = syn.analytic_vloc(3.0, 1.0)
    grid = D.DirectGrid(lat, (32, 32, 32))
    ions = D.Ions(symbols=["Al"] * 4, positions=pos, cell=lat)
    pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": D.functional.RECPOT(r=gp, v=vp, zval=3)}, PME=True)
    tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="GGA", k_str="LKT"),
                            XCFunctional=D.Functional(type="XC", name="LDA"),
                            HARTREE=D.Functional(type="HARTREE"), PSEUDO=pp)
    rho0 = D.DirectField(grid) + 12.0 / grid.volume
    opts = {"econv": 1e-6 * 4, "maxiter": 300, "maxfun": 50}
    opt = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS", optimization_options=dict(opts))
    rho = opt.optimize_rho(guess_rho=rho0)
    assert opt.converged == 0
    assert abs(float(rho.integral()) - 12.0) < 1e-9 * 12.0
    mix = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS", optimization_options=dict(opts))
    mix.optimize_rho_mixed(guess_rho=rho0, refine="optimize")
    # both stop at the econv rule (1e-6 Ha/atom per iteration), from different paths
    assert abs(mix.functional.energy - opt.functional.energy) / 4 <= 1e-5


@pytest.mark.parametrize("tag,name,sigma", [("VW_SIG", "vW", 0.2), ("TFVW_SIG", "TFVW", 0.35)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_vw_sigma_against_reference(golden, tag, name, sigma, dtype):
    """vW with the Laplacian smoothed by exp(-G^2 sigma^2/4) (vw.py:29-53)."""
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"], dtype=dtype)
    o = D.Functional(type="KEDF", name=name, sigma=sigma)(rho)
    e, v = GG["A_E_" + tag], GG["A_V_" + tag]
    tol = (1e-10, 1e-9) if dtype == torch.float64 else (2e-6, 1e-4)
    assert abs(o.energy - e) <= tol[0] * abs(e), (o.energy, e)
    assert float(np.abs(_np(o.potential) - v).max()) <= tol[1] * float(np.abs(v).max())


def test_gga_sigma_fp32():
    grid = D.DirectGrid(np.diag([15.2, 15.2, 15.2]), (64, 64, 64))
    rho_np = syn.smooth_density(grid.lattice, (64, 64, 64), 32.0, seed=12, amp=0.5)
    out = {}
    for dt in (torch.float64, torch.float32):
        o = D.Functional(type="KEDF", name="GGA", k_str="LKT", sigma=0.3)(D.DirectField(grid, data=rho_np, dtype=dt))
        out[dt] = (o.energy, _np(o.potential))
    (e64, v64), (e32, v32) = out[torch.float64], out[torch.float32]
    assert abs(e32 - e64) <= 2e-6 * abs(e64)
    assert float(np.abs(v32 - v64).max()) <= 1e-4 * float(np.abs(v64).max())


MCASES = [(str(n), str(n), {}) for n in GG["mgga_names"]] + [("PGSL_SIG", "PGSL", {"sigma": 0.3}),
                                                            ("GE4_P", "GE4", {"params": [1.0, 0.2, 2.0]}),
                                                            ("PGSL_RVW", "PGSL", {"gga_remove_vw": 0.5})]


@pytest.mark.parametrize("tag,name,kw", MCASES, ids=[c[0] for c in MCASES])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_mgga_against_reference(golden, tag, name, kw, dtype):
    """Meta-GGA (MGGA_<name>, gga.py:1226-1308): energy and potential; FP32 within
    2e-6 relative and 1e-4 of max|V|."""
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"], dtype=dtype)
    f = D.Functional(type="KEDF", name="MGGA_" + name, **kw)
    o = f(rho)
    e, v = GG["A_E_M" + tag], GG["A_V_M" + tag]
    tol = (1e-10, 1e-9) if dtype == torch.float64 else (2e-6, 1e-4)
    assert abs(o.energy - e) <= tol[0] * abs(e), (o.energy, e)
    assert float(np.abs(_np(o.potential) - v).max()) <= tol[1] * float(np.abs(v).max())
    if dtype == torch.float64:
        with pytest.raises(AttributeError):
            f.stress(rho)


@pytest.mark.parametrize("tag,kw", [("LKTE", {}), ("LKTE_P", {"params": [1.1]}), ("LKTE_S", {"sigma": 0.2, "y": 0.9})])
def test_lkt_engine_against_reference(golden, tag, kw):
    """KEDF 'LKT' (lkt.py): GGA 'LKT-VW' plus vW in one fused evaluation."""
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    o = D.Functional(type="KEDF", name="LKT", **kw)(rho)
    e, v = GG["A_E_" + tag], GG["A_V_" + tag]
    assert abs(o.energy - e) <= 1e-10 * abs(e), (o.energy, e)
    assert float(np.abs(_np(o.potential) - v).max()) <= 1e-9 * float(np.abs(v).max())
