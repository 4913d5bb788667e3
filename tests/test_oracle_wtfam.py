"""The Smargiassi-Madden and Perrot kinetic functionals (kedf/sm.py, fp.py: the
WT engine with alpha = beta = 1/2 and 1) restated with the oracle's WT term,
against the reference's outputs (tests/golden/make_golden_wtfam.py); the SM
stress takes alpha = beta = 1 unless given (sm.py:18-19)."""
import os

import numpy as np
import pytest

from oracle import ofdft_np as O

HERE = os.path.dirname(os.path.abspath(__file__))
WF = dict(np.load(os.path.join(HERE, "golden", "reference_wtfam.npz")))
# tag -> (local terms, energy exponent, stress exponent)
CASES = {"SM": (True, 0.5, 1.0), "FP": (True, 1.0, 1.0), "SMNL": (False, 0.5, 1.0), "SMA": (True, 0.6, 0.6)}


@pytest.mark.parametrize("tag", sorted(CASES))
def test_wt_family(golden, tag):
    local, a, a_s = CASES[tag]
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    rho = golden["A_rho"]
    nl = O.WT(alpha=a, beta=a)(rho, grid)
    E, V = nl["E"], nl["V"]
    S = O.wt_stress(rho, grid, nl["E"], alpha=a_s, beta=a_s)
    if local:
        t, w = O.tf(rho, grid), O.vw(rho, grid)
        E, V = E + t["E"] + w["E"], V + t["V"] + w["V"]
        S = S + O.tf_stress(grid, t["E"]) + O.vw_stress(rho, grid)
    assert abs(E - WF["A_E_" + tag]) <= 1e-11 * abs(E)
    np.testing.assert_allclose(V, WF["A_V_" + tag], rtol=0, atol=1e-10 * np.abs(V).max())
    np.testing.assert_allclose(S, WF["A_S_" + tag], rtol=0, atol=1e-10 * np.abs(S).max())


@pytest.mark.parametrize("tag,local,kw", [("WTE", True, {}), ("WTENL", False, {}),
                                          ("WTEX", True, {"x": 0.8, "alpha": 0.9, "beta": 0.7})])
def test_wte(golden, tag, local, kw):
    """WTE (wte.py:15-57): E_TF exp(E_WT/E_TF), its potential and stress, plus vW for 'WTE'."""
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    rho = golden["A_rho"]
    x, a, b = kw.get("x", 1.0), kw.get("alpha", 5.0 / 6.0), kw.get("beta", 5.0 / 6.0)
    t = O.tf(rho, grid, x=x)
    w = O.WT(x=x, alpha=a, beta=b)(rho, grid)
    r = w["E"] / t["E"]
    E = t["E"] * np.exp(r)
    V = np.exp(r) * ((1 - r) * t["V"] + w["V"])
    S = O.wt_stress(rho, grid, w["E"], alpha=a, beta=b) + np.eye(3) * (2.0 / 3.0 * w["E"] / grid.volume)
    S = (S + O.tf_stress(grid, t["E"])) * np.exp(r)
    if local:
        vw = O.vw(rho, grid)
        E, V, S = E + vw["E"], V + vw["V"], S + O.vw_stress(rho, grid)
    assert abs(E - WF["A_E_" + tag]) <= 1e-11 * abs(E)
    np.testing.assert_allclose(V, WF["A_V_" + tag], rtol=0, atol=1e-10 * np.abs(V).max())
    np.testing.assert_allclose(S, WF["A_S_" + tag], rtol=0, atol=1e-10 * np.abs(S).max())


MGP_ORACLE = {"MGP": (True, {}), "MGPA": (True, {"symmetrization": "Arithmetic"}),
              "MGPG": (True, {"symmetrization": "Geometric"}), "MGP0": (True, {"revke": False}),
              # KEDF drops options set to None (kedf/__init__.py:144), so the lump default 0.2 stays
              "MGPNL": (False, {"maxpoint": 200}),
              "MGP0L": (True, {"revke": False, "lumpfactor": [0.1, 0.3, 2.0]}),
              "MGPS": (True, {"symmetrization": "Geometric"})}


@pytest.mark.parametrize("tag", sorted(MGP_ORACLE))
def test_mgp(golden, tag):
    """The density-independent MGP kernels (mgp.py:15-119), E and V."""
    local, kw = MGP_ORACLE[tag]
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    rho = golden["A_rho"]
    nl = O.MGP(**kw)(rho, grid)
    E, V = nl["E"], nl["V"]
    if local:
        t, w = O.tf(rho, grid), O.vw(rho, grid)
        E, V = E + t["E"] + w["E"], V + t["V"] + w["V"]
    assert abs(E - WF["A_E_" + tag]) <= 1e-11 * abs(E)
    np.testing.assert_allclose(V, WF["A_V_" + tag], rtol=0, atol=1e-10 * np.abs(V).max())


TTF_ORACLE = {"TTF1": (("TF", "VW"), {}, 0.5, False, 1.0), "TTF2": (("TF",), {}, 1.2, False, 0.9),
              "TTF0": (("TF", "VW"), {}, 0.5, True, 1.0), "TTFW": (("TF", "VW", "WT"), {}, 0.05, False, 1.0)}


@pytest.mark.parametrize("tag", sorted(TTF_ORACLE))
def test_ttf(golden, tag):
    """A temperature option adds TTF (tf.py:83-204) to the KEDF."""
    names, _, T, old, x = TTF_ORACLE[tag]
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    rho = golden["A_rho"]
    d = O.ttf(rho, grid, T, x=x, old=old)
    assert abs(d["E"] - WF["A_EDTTF_" + tag]) <= 1e-11 * abs(d["E"])
    E, V = d["E"], d["V"]
    for n in names:
        o = {"TF": lambda: O.tf(rho, grid, x=x), "VW": lambda: O.vw(rho, grid), "WT": lambda: O.WT()(rho, grid)}[n]()
        E, V = E + o["E"], V + o["V"]
    assert abs(E - WF["A_E_" + tag]) <= 1e-11 * abs(E)
    np.testing.assert_allclose(V, WF["A_V_" + tag], rtol=0, atol=1e-10 * np.abs(V).max())
