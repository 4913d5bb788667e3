"""GPU parity of the Fourier interpolation between grids (grid_map_data,
field2distrib; utils/utils.py:50-285) against the reference's outputs
(tests/golden/make_golden_gridmap.py), and the multi-step optimisation of
OptimizeDensityConf (interface.py:183-205) built on it.

Bars: FP64 within 1e-14 of max|rho|, FP32 within 1e-6."""
import os
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn
from dftpy_gb300.utils import field2distrib, grid_map_data

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden_gridmap import LAT, NR, TARGETS, source_density  # noqa: E402

GM = dict(np.load(os.path.join(HERE, "golden", "reference_gridmap.npz")))


def _np(f):
    return f.as_subclass(torch.Tensor).double().cpu().numpy()


@pytest.mark.parametrize("nr", TARGETS, ids=["x".join(map(str, t)) for t in TARGETS])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_grid_map_against_reference(nr, dtype):
    rho = D.DirectField(D.DirectGrid(LAT, NR), data=source_density(), dtype=dtype)
    out = grid_map_data(rho, nr)
    ref = GM["map_" + "x".join(map(str, nr))]
    assert out.shape == ref.shape and out.dtype == dtype and tuple(out.grid.nrR) == tuple(nr)
    tol = 1e-14 if dtype == torch.float64 else 1e-6
    assert float(np.abs(_np(out) - ref).max()) <= tol * np.abs(ref).max()


def test_field2distrib_against_reference():
    f = source_density()
    src = D.DirectField(D.DirectGrid(LAT, NR), data=f - 0.8 * f.mean())
    dst = D.DirectField(D.DirectGrid(LAT, (15, 13, 11)))
    field2distrib(src, dst, root=0)
    ref = GM["distrib_15x13x11"]
    assert float(np.abs(_np(dst) - ref).max()) <= 1e-14 * np.abs(ref).max()
    assert int((_np(dst) == 1e-30).sum()) == int((ref == 1e-30).sum())


def test_multistep_optimize_density_conf():
    """MATH.multistep = 2: the ground state on 24^3, interpolated to 48^3 and
    re-optimised there, reaches the 48^3 ground state from the uniform density."""
    from dftpy_gb300.interface import OptimizeDensityConf
    lat, pos = syn.fcc_cell(7.6)
    gp, vp = syn.analytic_vloc(3.0, 1.0)

    def system(n):
        grid = D.DirectGrid(lat, (n, n, n))
        ions = D.Ions(symbols=["Al"] * 4, positions=pos, cell=lat)
        pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": D.functional.RECPOT(r=gp, v=vp, zval=3)}, PME=True)
        tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="WT"),
                                XCFunctional=D.Functional(type="XC", name="LDA"),
                                HARTREE=D.Functional(type="HARTREE"), PSEUDO=pp)
        return grid, ions, tot, D.DirectField(grid) + 12.0 / grid.volume

    grid, ions, tot, rho0 = system(24)
    cfg = {"OPT": {"method": "LBFGS", "econv": 1e-9, "maxiter": 300}, "MATH": {"multistep": 2},
           "JOB": {"calctype": "Energy"}}
    res = OptimizeDensityConf(cfg, ions=ions, rho=rho0, E_v_Evaluator=tot)
    rho = res["density"]
    assert tuple(rho.grid.nrR) == (48, 48, 48)
    assert abs(float(rho.integral()) - 12.0) <= 1e-9 * 12
    grid2, ions2, tot2, rho02 = system(48)
    opt = D.Optimization(EnergyEvaluator=tot2, optimization_method="LBFGS",
                         optimization_options={"econv": 1e-9 * 4, "maxiter": 300})
    opt.optimize_rho(guess_rho=rho02)
    assert abs(res["energypotential"]["TOTAL"].energy - opt.functional.energy) <= 1e-7 * 4


def test_electrostatic_potential_and_outputs(tmp_path):
    """get_electrostatic_potential (properties/potential.py:3-7) is v_loc + v_H, and
    OptimizeDensityConf writes it and the density when DENSITY.densityoutput and
    OUTPUT.electrostatic_potential name files."""
    from dftpy_gb300 import formats as F
    from dftpy_gb300.interface import OptimizeDensityConf
    from dftpy_gb300.properties import get_electrostatic_potential
    lat, pos = syn.fcc_cell(7.6)
    gp, vp = syn.analytic_vloc(3.0, 1.0)
    grid = D.DirectGrid(lat, (24, 24, 24))
    ions = D.Ions(symbols=["Al"] * 4, positions=pos, cell=lat)
    pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": D.functional.RECPOT(r=gp, v=vp, zval=3)}, PME=True)
    ha = D.Functional(type="HARTREE")
    tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="TFVW"),
                            XCFunctional=D.Functional(type="XC", name="LDA"), HARTREE=ha, PSEUDO=pp)
    rho0 = D.DirectField(grid) + 12.0 / grid.volume
    fd, fv = str(tmp_path / "rho.xsf"), str(tmp_path / "ves.xsf")
    cfg = {"OPT": {"method": "LBFGS", "econv": 1e-8}, "DENSITY": {"densityoutput": fd},
           "OUTPUT": {"electrostatic_potential": fv}}
    res = OptimizeDensityConf(cfg, ions=ions, rho=rho0, E_v_Evaluator=tot)
    rho = res["density"]
    v = get_electrostatic_potential(rho, tot)
    ref = pp(rho, calcType={"V"}).potential.as_subclass(torch.Tensor) + ha(rho, calcType={"V"}).potential.as_subclass(
        torch.Tensor)
    assert torch.allclose(v.as_subclass(torch.Tensor), ref, rtol=0, atol=1e-14)
    back_v, back_rho = F.read_density(fv), F.read_density(fd)
    assert float(np.abs(_np(back_v) - _np(v)).max()) <= 1e-12 * float(np.abs(_np(v)).max())
    assert float(np.abs(_np(back_rho) - _np(rho)).max()) <= 1e-12 * float(np.abs(_np(rho)).max())
