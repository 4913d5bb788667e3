"""The oracle's density mixers and OE-SCF (oracle/ofdft_np.py) against the
reference's outputs (tests/golden/make_golden_scf.py): Pulay and linear mixing
with every preconditioner, the high-frequency cutoff, history roll-over and
restarts; the preconditioner called directly; the external-potential energy;
and the OE-SCF energy history and density."""
import os
import sys

import numpy as np

from oracle import ofdft_np as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden_scf import MIX_CASES, MIX_LAT, MIX_NR, MIX_STEPS, mix_inputs  # noqa: E402

SG = dict(np.load(os.path.join(HERE, "golden", "reference_scf.npz")))


def test_mixers_match_reference():
    grid = O.Grid(MIX_LAT, MIX_NR)
    nin0, Q = mix_inputs()
    for tag, scheme, kw in MIX_CASES:
        m = O.PulayMixer(grid, **kw) if scheme == "pulay" else O.LinearMixer(grid, **kw)
        nin = nin0.copy()
        for k in range(MIX_STEPS):
            nin = m(nin, 0.9 * nin + 0.1 * Q[k])
        ref = SG["mix_" + tag + "_final"]
        assert np.abs(nin - ref).max() <= 1e-13 * np.abs(ref).max(), tag


def test_precondition_direct():
    grid = O.Grid(MIX_LAT, MIX_NR)
    nin0, Q = mix_inputs()
    drho = 0.05 * (Q[1] - Q[2])
    res = 0.3 * (Q[3] - nin0)
    a = O.precondition(nin0, Q[0], grid, "kerker", [0.9, 1.1, 0.7], 3.0, drho=drho, residual=res, coef=0.45)
    np.testing.assert_allclose(a, SG["pred_direct"], rtol=0, atol=1e-14)
    b = O.precondition(nin0, Q[0], grid, "kerker", [0.9, 1.1, 0.7], 3.0, residual=res)
    np.testing.assert_allclose(b, SG["pred_resonly"], rtol=0, atol=1e-14)


def test_external_energy():
    from dftpy_gb300 import synthetic as syn
    grid = O.Grid(MIX_LAT, MIX_NR)
    nin0, _ = mix_inputs()
    v = syn.smooth_density(MIX_LAT, MIX_NR, 3.0, seed=50, amp=0.6) - 0.2
    assert abs((v * nin0).sum() * grid.dV - SG["ext_E"]) <= 1e-13 * abs(SG["ext_E"])


def test_oescf_matches_reference(golden):
    grid = O.Grid(SG["scf_lattice"], (24, 24, 24))
    pp = O.LocalPseudo(grid, SG["scf_pos"], np.zeros(4, dtype=int), [(golden["recpot_gp"], golden["recpot_vp"])],
                       PME=True)
    terms = O.make_terms(grid, "VW", pseudo=pp)
    emb = O.make_terms(grid, "WT", xc=False, hartree=False, y=0.0)
    rho0 = np.full(tuple(grid.nr), 12.0 / grid.volume)
    mixer = O.PulayMixer(grid, predtype="kerker", predcoef=[1.0, 1.0, 1.0], maxm=7, coef=0.7, delay=2)
    ew = O.Ewald(grid, SG["scf_pos"], np.full(4, 3.0), PME=True)
    rho, info = O.oescf(terms, emb, rho0, grid, mixer, econv=1e-6 * 4, maxiter=100, method="CG-HS",
                        ewald_energy=ew.energy())
    h = np.array(info["history"])
    ref = SG["scf_energy_history"]
    assert info["iter"] == int(SG["scf_iter"])
    np.testing.assert_allclose(h, ref, rtol=1e-10, atol=0)
    # the inner optimisations stop at loose thresholds, so rounding differences
    # show in the density at the 1e-7 level while the energies agree to 1e-10
    assert np.abs(rho - SG["scf_rho"]).max() <= 1e-6 * np.abs(SG["scf_rho"]).max()
