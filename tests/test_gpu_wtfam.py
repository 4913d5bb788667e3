"""GPU parity of the Smargiassi-Madden and Perrot kinetic functionals (kedf/sm.py,
fp.py) and of WTE (wte.py) against the reference's outputs (tests/golden/make_golden_wtfam.py):
energy within 1e-10 relative, potential within 1e-9 and stress within 1e-9 of
their largest values in FP64; FP32 energy within 2e-6 relative."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D

HERE = os.path.dirname(os.path.abspath(__file__))
WF = dict(np.load(os.path.join(HERE, "golden", "reference_wtfam.npz")))
CASES = [("SM", "SM", {}), ("FP", "FP", {}), ("SMNL", "SM-NL", {}), ("SMA", "SM", {"alpha": 0.6, "beta": 0.6}),
         ("WTE", "WTE", {}), ("WTENL", "WTE-NL", {}), ("WTEX", "WTE", {"x": 0.8, "alpha": 0.9, "beta": 0.7})]


def _np(f):
    return f.as_subclass(torch.Tensor).double().cpu().numpy()


@pytest.mark.parametrize("tag,name,kw", CASES, ids=[c[0] for c in CASES])
def test_wt_family_against_reference(golden, tag, name, kw):
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    f = D.Functional(type="KEDF", name=name, **kw)
    o = f(rho)
    e, v, s = WF["A_E_" + tag], WF["A_V_" + tag], WF["A_S_" + tag]
    assert abs(o.energy - e) <= 1e-10 * abs(e), (o.energy, e)
    assert float(np.abs(_np(o.potential) - v).max()) <= 1e-9 * min(1.0, float(np.abs(v).max()))
    st = f.stress(rho)
    assert float(np.abs(st - s).max()) <= 1e-9 * float(np.abs(s).max())
    o32 = f(D.DirectField(grid, data=golden["A_rho"], dtype=torch.float32))
    assert abs(o32.energy - e) <= 2e-6 * abs(e)


def test_wte_ground_state():
    """WTE in a fused total functional drives the native optimiser; at its ground
    state the potential is flat up to the chemical potential."""
    from dftpy_gb300 import synthetic as syn
    lat, pos = syn.fcc_cell(7.6)
    gp, vp = syn.analytic_vloc(3.0, 1.0)
    grid = D.DirectGrid(lat, (24, 24, 24))
    ions = D.Ions(symbols=["Al"] * 4, positions=pos, cell=lat)
    pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": D.functional.RECPOT(r=gp, v=vp, zval=3)}, PME=True)
    tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="WTE"),
                            XCFunctional=D.Functional(type="XC", name="LDA"), HARTREE=D.Functional(type="HARTREE"),
                            PSEUDO=pp)
    opt = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS",
                         optimization_options={"econv": 1e-9 * 4, "maxiter": 300})
    rho = opt.optimize_rho(guess_rho=D.DirectField(grid) + 12.0 / grid.volume)
    assert opt.converged == 0
    v = _np(opt.functional.potential)
    r = _np(rho)
    assert np.abs((v - opt.mu) * np.sqrt(r)).max() < 1e-3


MGP_CASES = [("MGP", "MGP", {}), ("MGPA", "MGPA", {}), ("MGPG", "MGPG", {}), ("MGP0", "MGP0", {}),
             ("MGPNL", "MGP-NL", {"maxpoint": 200, "lumpfactor": None}),
             ("MGP0L", "MGP0", {"lumpfactor": [0.1, 0.3, 2.0]}), ("MGPS", "MGP", {"symmetrization": "Geometric"})]


@pytest.mark.parametrize("tag,name,kw", MGP_CASES, ids=[c[0] for c in MGP_CASES])
def test_mgp_against_reference(golden, tag, name, kw):
    """The MGP kernels at rho0 (mgp.py:15-119), the t integral evaluated on the device."""
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    f = D.Functional(type="KEDF", name=name, **kw)
    o = f(rho)
    e, v = WF["A_E_" + tag], WF["A_V_" + tag]
    assert abs(o.energy - e) <= 1e-10 * abs(e), (o.energy, e)
    assert float(np.abs(_np(o.potential) - v).max()) <= 1e-9 * min(1.0, float(np.abs(v).max()))
    o32 = f(D.DirectField(grid, data=golden["A_rho"], dtype=torch.float32))
    assert abs(o32.energy - e) <= 2e-6 * abs(e)
    with pytest.raises(AttributeError):
        f.stress(rho)


TTF_CASES = [("TTF1", "TFVW", {"temperature": 0.5}), ("TTF2", "TF", {"temperature": 1.2, "x": 0.9}),
             ("TTF0", "TFVW", {"temperature0": 0.5}), ("TTFW", "WT", {"temperature": 0.05})]


@pytest.mark.parametrize("tag,name,kw", TTF_CASES, ids=[c[0] for c in TTF_CASES])
def test_ttf_against_reference(golden, tag, name, kw):
    """A temperature option adds the finite-temperature TF correction (tf.py:83-204);
    split=True reports it as 'DTTF' (kedf/__init__.py:155-156)."""
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    f = D.Functional(type="KEDF", name=name, **kw)
    o = f(rho)
    e, v = WF["A_E_" + tag], WF["A_V_" + tag]
    assert abs(o.energy - e) <= 1e-10 * abs(e), (o.energy, e)
    assert float(np.abs(_np(o.potential) - v).max()) <= 1e-9 * min(1.0, float(np.abs(v).max()))
    parts = f(rho, split=True)
    assert abs(parts["DTTF"].energy - WF["A_EDTTF_" + tag]) <= 1e-10 * abs(WF["A_EDTTF_" + tag])
    o32 = f(D.DirectField(grid, data=golden["A_rho"], dtype=torch.float32))
    assert abs(o32.energy - e) <= 2e-6 * abs(e)
