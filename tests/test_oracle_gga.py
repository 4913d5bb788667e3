"""Pin the oracle's GGA kinetic functionals against the reference's outputs
(tests/golden/make_golden_gga.py): every functional of the reference's list,
energy, potential and stress, plus the reference's own 'lc94' test."""
import os

import numpy as np
import pytest

from oracle import ofdft_np as O

HERE = os.path.dirname(os.path.abspath(__file__))
GG = dict(np.load(os.path.join(HERE, "golden", "reference_gga.npz")))
CASES = [(n, n, {}) for n in GG["names"]] + [("LKT_P", "LKT", {"params": [1.1, 0.9]}),
                                             ("LKT_RVW", "LKT", {"gga_remove_vw": 1.0}),
                                             ("LKT_SIG", "LKT", {"sigma": 0.2}), ("LC94_SIG", "LC94", {"sigma": 0.35})]


@pytest.mark.parametrize("tag,name,kw", CASES, ids=[c[0] for c in CASES])
def test_gga_system_a(golden, tag, name, kw):
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    r = O.gga(golden["A_rho"], grid, name, calc=("E", "V", "S"), **kw)
    e = GG["A_E_" + tag]
    assert abs(r["E"] - e) <= 1e-11 * max(1.0, abs(e)), (r["E"], e)
    v = GG["A_V_" + tag]
    np.testing.assert_allclose(r["V"], v, rtol=0, atol=1e-10 * max(1.0, np.abs(v).max()))
    s = GG["A_S_" + tag]
    np.testing.assert_allclose(r["S"], s, rtol=0, atol=1e-10 * max(1e-12, np.abs(s).max()))


def test_gga_reference_fixture(golden):
    grid = O.Grid(golden["E_lattice"], golden["E_nr"])
    e = O.gga(golden["E_rho"], grid, "LC94", calc=("E",))["E"]
    assert abs(e - GG["fixture_E_LC94"]) <= 1e-12 * abs(e)
    assert np.isclose(e, 1.6821337114254904)  # the reference's own test value


@pytest.mark.parametrize("tag,name,sigma", [("VW_SIG", "VW", 0.2), ("TFVW_SIG", "TFVW", 0.35)])
def test_vw_sigma(golden, tag, name, sigma):
    """The vW term with the Gaussian-smoothed Laplacian (vw.py:29-53)."""
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    rho = golden["A_rho"]
    r = O.vw(rho, grid, sigma=sigma)
    e, v = r["E"], r["V"]
    if name == "TFVW":
        t = O.tf(rho, grid)
        e, v = e + t["E"], v + t["V"]
    assert abs(e - GG["A_E_" + tag]) <= 1e-11 * abs(e)
    np.testing.assert_allclose(v, GG["A_V_" + tag], rtol=0, atol=1e-10 * np.abs(v).max())


MCASES = [(str(n), str(n), {}) for n in GG["mgga_names"]] + [("PGSL_SIG", "PGSL", {"sigma": 0.3}),
                                                            ("GE4_P", "GE4", {"params": [1.0, 0.2, 2.0]}),
                                                            ("PGSL_RVW", "PGSL", {"gga_remove_vw": 0.5})]


@pytest.mark.parametrize("tag,name,kw", MCASES, ids=[c[0] for c in MCASES])
def test_mgga_system_a(golden, tag, name, kw):
    """The Laplacian-level functionals (gga.py:492-545, 645-650), E and V."""
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    r = O.gga(golden["A_rho"], grid, name, mgga=True, **kw)
    e = GG["A_E_M" + tag]
    assert abs(r["E"] - e) <= 1e-11 * abs(e)
    v = GG["A_V_M" + tag]
    np.testing.assert_allclose(r["V"], v, rtol=0, atol=1e-10 * np.abs(v).max())


@pytest.mark.parametrize("tag,kw", [("LKTE", {}), ("LKTE_P", {"params": [1.1]}), ("LKTE_S", {"sigma": 0.2, "y": 0.9})])
def test_lkt_engine(golden, tag, kw):
    """The LKT engine (lkt.py): GGA 'LKT-VW' plus vW, sigma passed to both."""
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    rho = golden["A_rho"]
    g = O.gga(rho, grid, "LKT-VW", params=kw.get("params"), sigma=kw.get("sigma"))
    w = O.vw(rho, grid, y=kw.get("y", 1.0), sigma=kw.get("sigma"))
    E, V = g["E"] + w["E"], g["V"] + w["V"]
    assert abs(E - GG["A_E_" + tag]) <= 1e-11 * abs(E)
    np.testing.assert_allclose(V, GG["A_V_" + tag], rtol=0, atol=1e-10 * np.abs(V).max())
