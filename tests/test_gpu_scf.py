"""GPU parity of the density mixers, the external potential and the OE-SCF
solver (mixer/*.py, functional/external_potential.py, optimization/scf.py)
against the reference's outputs (tests/golden/make_golden_scf.py), through
the native library.

Bars: mixed densities after nine steps within 1e-11 of max|rho| (the device
transforms round differently from numpy's); the external energy within 1e-12
relative; the OE-SCF energy history within 1e-9 relative, the same number of
outer iterations, and the density within 1e-6 of max|rho| (the inner
optimisations stop at loose thresholds)."""
import os
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn
from dftpy_gb300.mixer import Mixer, SpecialPrecondition
from dftpy_gb300.optimization import OESCF

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden_scf import MIX_CASES, MIX_LAT, MIX_NR, MIX_STEPS, mix_inputs  # noqa: E402

SG = dict(np.load(os.path.join(HERE, "golden", "reference_scf.npz")))


def _np(f):
    return f.as_subclass(torch.Tensor).double().cpu().numpy()


@pytest.mark.parametrize("tag,scheme,kw", MIX_CASES, ids=[c[0] for c in MIX_CASES])
def test_mixer_against_reference(tag, scheme, kw):
    grid = D.DirectGrid(MIX_LAT, MIX_NR)
    nin0, Q = mix_inputs()
    mixer = Mixer(scheme=scheme, nspin=1, **kw)
    nin = D.DirectField(grid, data=nin0)
    Qd = [D.DirectField(grid, data=q) for q in Q]
    for k in range(MIX_STEPS):
        nout = 0.9 * nin + 0.1 * Qd[k]
        nin = mixer(nin, nout)
        assert nin.is_cuda and isinstance(nin, D.DirectField)
    ref = SG["mix_" + tag + "_final"]
    assert float(np.abs(_np(nin) - ref).max()) <= 1e-11 * np.abs(ref).max()


def test_mixer_fp32_against_fp64():
    grid = D.DirectGrid(MIX_LAT, MIX_NR)
    nin0, Q = mix_inputs()
    out = {}
    for dt in (torch.float64, torch.float32):
        mixer = Mixer(scheme="pulay", nspin=1, predtype="kerker", predcoef=[1.0, 1.0, 1.0], maxm=3, delay=1,
                      predecut=1.0)
        nin = D.DirectField(grid, data=nin0, dtype=dt)
        for k in range(MIX_STEPS):
            nin = mixer(nin, 0.9 * nin + 0.1 * D.DirectField(grid, data=Q[k], dtype=dt))
        out[dt] = _np(nin)
    assert np.abs(out[torch.float32] - out[torch.float64]).max() <= 1e-5 * np.abs(out[torch.float64]).max()


def test_precondition_direct():
    grid = D.DirectGrid(MIX_LAT, MIX_NR)
    nin0, Q = mix_inputs()
    pred = SpecialPrecondition("kerker", [0.9, 1.1, 0.7], predecut=3.0)
    nin, nout = D.DirectField(grid, data=nin0), D.DirectField(grid, data=Q[0])
    drho = D.DirectField(grid, data=0.05 * (Q[1] - Q[2]))
    res = D.DirectField(grid, data=0.3 * (Q[3] - nin0))
    a = pred(nin, nout, drho=drho, residual=res, coef=0.45)
    np.testing.assert_allclose(_np(a), SG["pred_direct"], rtol=0, atol=1e-13)
    b = pred(nin, nout, residual=res)
    np.testing.assert_allclose(_np(b), SG["pred_resonly"], rtol=0, atol=1e-13)


def test_external_potential():
    grid = D.DirectGrid(MIX_LAT, MIX_NR)
    nin0, _ = mix_inputs()
    v = syn.smooth_density(MIX_LAT, MIX_NR, 3.0, seed=50, amp=0.6) - 0.2
    ext = D.functional.ExternalPotential(v=D.DirectField(grid, data=v))
    rho = D.DirectField(grid, data=nin0)
    e = ext(rho, calcType={"E"}).energy
    assert abs(e - SG["ext_E"]) <= 1e-12 * abs(SG["ext_E"])
    # fused into a total functional: energies and potentials add
    xc = D.Functional(type="XC", name="LDA")
    tot = D.TotalFunctional(XC=xc, EXT=ext)
    o = tot(rho)
    oxc = xc(rho)
    assert abs(o.energy - (oxc.energy + e)) <= 1e-12 * abs(o.energy)
    np.testing.assert_allclose(_np(o.potential), _np(oxc.potential) + v, rtol=0, atol=1e-13)


def _scf_system(golden):
    lat, pos = SG["scf_lattice"], SG["scf_pos"]
    grid = D.DirectGrid(lat, (24, 24, 24))
    ions = D.Ions(symbols=["Al"] * 4, positions=pos, cell=lat)
    pp = D.LocalPseudo(grid=grid, ions=ions, PME=True,
                       PP_list={"Al": D.functional.RECPOT(r=golden["recpot_gp"], v=golden["recpot_vp"], zval=3)})
    xc = D.Functional(type="XC", name="LDA")
    ha = D.Functional(type="HARTREE")
    ee = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="vW"), XCFunctional=xc,
                           HARTREE=ha, PSEUDO=pp)
    emb = D.TotalFunctional(KEDF_EMB=D.Functional(type="KEDF", name="WT", y=0.0))
    rho0 = D.DirectField(grid) + 12.0 / grid.volume
    return grid, ions, pp, ee, emb, rho0


def test_oescf_against_reference(golden):
    grid, ions, pp, ee, emb, rho0 = _scf_system(golden)
    opt = D.Optimization(EnergyEvaluator=ee, optimization_method="CG-HS",
                         optimization_options={"econv": 1e-6 * 4, "maxiter": 100})
    mixer = Mixer(scheme="pulay", nspin=1, predtype="kerker", predcoef=[1.0, 1.0, 1.0], maxm=7, coef=0.7, delay=2)
    sc = OESCF(optimization=opt, evaluator_emb=emb, mixer=mixer)
    rho = sc.optimize_rho(guess_rho=rho0)
    assert sc.converged and sc.iter == int(SG["scf_iter"])
    np.testing.assert_allclose(np.array(sc.energyhistory), SG["scf_energy_history"], rtol=1e-9, atol=0)
    ref = SG["scf_rho"]
    assert float(np.abs(_np(rho) - ref).max()) <= 1e-6 * np.abs(ref).max()
    assert "EMB" not in ee.funcDict
    assert abs(opt.optimization_options["econv"] - SG["scf_econv_final"]) <= 1e-12 * SG["scf_econv_final"]


def test_optimize_density_conf(golden):
    """OptimizeDensityConf (interface.py:150-229) with OPT.algorithm OESCF: the
    same OE-SCF run, then the energy of the full functional (vW + the
    embedding KEDF) on its density."""
    from dftpy_gb300.interface import OptimizeDensityConf
    grid, ions, pp, ee, emb, rho0 = _scf_system(golden)
    config = {"OPT": {"algorithm": "OESCF", "method": "CG-HS", "econv": 1e-6},
              "MIX": {"scheme": "pulay", "predtype": "kerker", "predcoef": [1.0, 1.0, 1.0], "maxm": 7,
                      "coef": 0.7, "delay": 2},
              "JOB": {"task": "Optdensity", "calctype": "Energy"}}
    res = OptimizeDensityConf(config, ions=ions, rho=rho0, E_v_Evaluator=ee, evaluator_emb=emb)
    rho = res["density"]
    assert float(np.abs(_np(rho) - SG["scf_rho"]).max()) <= 1e-6 * np.abs(SG["scf_rho"]).max()
    full = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="WT"),
                             XCFunctional=D.Functional(type="XC", name="LDA"), HARTREE=D.Functional(type="HARTREE"),
                             PSEUDO=pp)
    e_full = full(rho, calcType={"E"}).energy
    assert abs(res["energypotential"]["TOTAL"].energy - e_full) <= 1e-10 * abs(e_full)
    assert "KEDF_EMB" not in ee.funcDict
    # direct optimisation through the same entry point (OPT.algorithm EMM)
    grid, ions, pp, ee, emb, rho0 = _scf_system(golden)
    res2 = OptimizeDensityConf({"OPT": {"econv": 1e-9}, "JOB": {"calctype": "Energy Force"}},
                               ions=ions, rho=rho0, E_v_Evaluator=full.__class__(
                                   KineticEnergyFunctional=D.Functional(type="KEDF", name="WT"),
                                   XCFunctional=D.Functional(type="XC", name="LDA"),
                                   HARTREE=D.Functional(type="HARTREE"), PSEUDO=pp))
    assert res2["forces"]["TOTAL"].shape == (4, 3)
    # OE-SCF converges (loosely) to the WT ground state
    assert abs(res2["energypotential"]["TOTAL"].energy - e_full) <= 1e-3 * 4
