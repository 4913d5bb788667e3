"""Pin the numpy oracle against golden vectors produced by the reference itself
(tests/golden/make_golden.py) and against the reference's own test goldens."""
import os
import tempfile

import numpy as np
import pytest

from oracle import ofdft_np as O

WGC = dict(alpha=(5 + np.sqrt(5)) / 6, beta=(5 - np.sqrt(5)) / 6)


def _close(a, b, rtol=1e-11, atol=1e-11):
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


def _fields(g, prefix, with_pp):
    lat, nr, rho = g[prefix + "lattice"], g[prefix + "nr"], g[prefix + "rho"]
    grid = O.Grid(lat, nr)
    res = {"TF": O.tf(rho, grid), "VW": O.vw(rho, grid), "XC": O.lda(rho, grid),
           "H": O.hartree(rho, grid), "WTNL": O.WT()(rho, grid)}
    if with_pp:
        gp, vp = g["recpot_gp"], g["recpot_vp"]
        pos = g[prefix + "pos"]
        sp = np.zeros(len(pos), dtype=int)
        res["PPPME"] = O.LocalPseudo(grid, pos, sp, [(gp, vp)], PME=True)(rho)
        res["PPEX"] = O.LocalPseudo(grid, pos, sp, [(gp, vp)], PME=False)(rho)
    return grid, rho, res


@pytest.mark.parametrize("prefix,with_pp", [("A_", True), ("B_", False)])
def test_local_and_fft_terms(golden, prefix, with_pp):
    grid, rho, res = _fields(golden, prefix, with_pp)
    for k, o in res.items():
        _close(o["E"], golden[prefix + "E_" + k], rtol=1e-12, atol=1e-12)
        vref = golden[prefix + "V_" + k]
        _close(o["V"], vref, rtol=0, atol=1e-10 * max(1.0, np.abs(vref).max()))


def test_pp_forces(golden):
    g = golden
    grid = O.Grid(g["A_lattice"], g["A_nr"])
    sp = np.zeros(len(g["A_pos"]), dtype=int)
    tab = [(g["recpot_gp"], g["recpot_vp"])]
    for pme, key in ((True, "A_F_PPPME"), (False, "A_F_PPEX")):
        F = O.LocalPseudo(grid, g["A_pos"], sp, tab, PME=pme).forces(g["A_rho"])
        _close(F, g[key], rtol=0, atol=1e-11)


@pytest.mark.parametrize("tag,kw", [
    ("A_LWT64", dict(nsp=64, kdd=3, interp="linear", **WGC)),
    ("A_LWT8H", dict(nsp=8, kdd=3, interp="hermite", **WGC)),
    ("A_LWTR", dict(ratio=1.15, kdd=3, interp="linear")),
    ("A_LWT8K1", dict(nsp=8, kdd=1, interp="linear", **WGC)),
    ("B_LWT16", dict(nsp=16, kdd=3, interp="linear", **WGC)),
    ("B_LWT6H", dict(nsp=6, kdd=3, interp="hermite")),
])
def test_lwt(golden, tag, kw):
    pre = tag[:2]
    grid = O.Grid(golden[pre + "lattice"], golden[pre + "nr"])
    rho = golden[pre + "rho"]
    o = O.LWT(**kw)(rho, grid)
    _close(o["E"], golden[pre + "E_" + tag[2:]], rtol=1e-11, atol=1e-12)
    vref = golden[pre + "V_" + tag[2:]]
    _close(o["V"], vref, rtol=0, atol=1e-9 * max(1.0, np.abs(vref).max()))


def test_ewald(golden):
    g = golden
    grid = O.Grid(g["A_lattice"], g["A_nr"])
    q = np.full(len(g["A_pos"]), 3.0)
    ew = O.Ewald(grid, g["A_pos"], q, PME=True)
    assert ew.eta == pytest.approx(float(g["A_ewald_eta"]), abs=1e-12)
    _close(ew.energy_corr(), g["A_ewald_Ecorr"])
    _close(ew.energy_real(), g["A_ewald_Ereal"], rtol=1e-11, atol=1e-11)
    _close(ew.energy_rec(), g["A_ewald_Erec"])
    _close(ew.energy(), g["A_ewald_E"])
    _close(ew.forces(), g["A_ewald_F"], rtol=0, atol=1e-10)
    ex = O.Ewald(grid, g["A_pos"], q, PME=False)
    _close(ex.energy(), g["A_ewaldex_E"])
    _close(ex.forces(), g["A_ewaldex_F"], rtol=0, atol=1e-10)


def test_two_species_pme(golden):
    g = golden
    grid = O.Grid(g["D_lattice"], g["D_nr"])
    tabs = [(g["recpot_gp"], g["recpot_vp"])]
    from dftpy_gb300.synthetic import analytic_vloc
    with tempfile.TemporaryDirectory() as d:
        gb, vb = analytic_vloc(2.0, 1.2)
        O.write_recpot(os.path.join(d, "b.recpot"), gb[-1], vb)
        gpb, vpb, zb = O.read_recpot(os.path.join(d, "b.recpot"))
    tabs.append((gpb, vpb))
    sp = g["D_species"]
    pp = O.LocalPseudo(grid, g["D_pos"], sp, tabs, PME=True)
    _close(pp(g["D_rho"])["E"], g["D_E_PP"])
    _close(pp.forces(g["D_rho"]), g["D_F_PP"], rtol=0, atol=1e-10)
    q = np.where(sp == 0, 3.0, 2.0)
    ew = O.Ewald(grid, g["D_pos"], q, PME=True)
    _close(ew.energy(), g["D_ewald_E"])
    _close(ew.forces(), g["D_ewald_F"], rtol=0, atol=1e-10)
    tot = sum(O.tf(g["D_rho"], grid).values()) if False else None
    wt = O.make_terms(grid, "WT", xc=False, hartree=False)
    e = sum(fn(g["D_rho"], ("E",))["E"] for _, fn in wt)
    _close(e, g["D_E_WT"])


def test_recpot_roundtrip(golden):
    with tempfile.TemporaryDirectory() as d:
        fn = os.path.join(d, "a.recpot")
        with open(fn, "wb") as f:
            f.write(golden["recpot_text"].tobytes())
        gp, vp, z = O.read_recpot(fn)
    np.testing.assert_array_equal(gp, golden["recpot_gp"])
    np.testing.assert_array_equal(vp, golden["recpot_vp"])
    assert z == golden["recpot_zval"] == 3


def test_reference_fixture_goldens(golden):
    """The reference's own test goldens (examples/test/test_functional.py:23-27,
    test_read_pp.py:10-31, test_ewald.py:11-53) on its Al_fde_rho.pp fixture."""
    g = golden
    grid = O.Grid(g["E_lattice"], g["E_nr"])
    rho = g["E_rho"]
    terms = O.make_terms(grid, "WT", xc=False, hartree=False)
    e = sum(fn(rho, ("E", "V"))["E"] for _, fn in terms)
    # reference golden 2.916818700014412 is on the reader's full complex grid; the
    # half grid differs on the Nyquist planes of this non-orthogonal cell by ~1e-3
    assert np.isclose(g["E_E_WT_fullgrid"], 2.916818700014412)
    assert np.isclose(e, 2.916818700014412, atol=2e-3)
    _close(e, g["E_E_WT"])
    sp = np.zeros(len(g["E_pos"]), dtype=int)
    pp = O.LocalPseudo(grid, g["E_pos"], sp, [(g["E_pp_al_gp"], g["E_pp_al_vp"])], PME=True)
    epp = pp(rho)["E"]
    assert np.isclose(epp, 1.3497046, atol=1e-4)
    _close(epp, g["E_E_PP_allda"])
    ew = O.Ewald(grid, g["E_pos"], np.full(len(g["E_pos"]), 3.0), PME=True)
    assert np.isclose(ew.energy_corr(), -13.003839613564997, atol=1e-5)
    assert np.isclose(ew.energy_rec(), 7.606943756474895, atol=1e-5)
    _close(ew.energy(), g["E_ewald_E"])
    _close(ew.forces(), g["E_ewald_F"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("method", ["TN", "LBFGS", "CGHS"])
def test_optimizer_c1(golden, method):
    g = golden
    from dftpy_gb300.synthetic import fcc_cell
    lat, pos = fcc_cell(7.60)
    grid = O.Grid(lat, (32, 32, 32))
    pp = O.LocalPseudo(grid, pos, np.zeros(4, dtype=int), [(g["recpot_gp"], g["recpot_vp"])], PME=True)
    ew = O.Ewald(grid, pos, np.full(4, 3.0), PME=True)
    _close(ew.energy(), g["C_ewald_E"])
    tot = O.Total(grid, O.make_terms(grid, "TFVW", pseudo=pp), ewald_energy=ew.energy())
    rho0 = np.full((32, 32, 32), 12.0 / grid.volume)
    m = {"TN": "TN", "LBFGS": "LBFGS", "CGHS": "CG-HS"}[method]
    rho, info = O.optimize(tot, rho0, grid, method=m, maxiter=60, maxfun=50, econv=1e-11 * 4)
    tag = "C_" + method + "_"
    assert info["converged"] == g[tag + "converged"] == 0
    _close(tot(rho, ("E",))["E"], g[tag + "E"], rtol=1e-11, atol=0)
    _close(info["mu"], g[tag + "mu"], rtol=1e-6, atol=0)
    if method == "TN":
        # the TN Hessian products use a 1e-9 finite difference, so iterates carry
        # ~1e-7 relative noise from summation order; the ground state agrees to ~1e-6
        np.testing.assert_allclose(rho, g["C_TN_rho"], rtol=2e-6, atol=0)


def test_golden_recipe_reproduces_edge_density(golden):
    """The committed generator pins the B block's input: its edge_density (plus
    the two planted values) gives the stored B_rho bit for bit."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    rho = mg.edge_density(golden["B_lattice"], tuple(golden["B_nr"]), np.array([[1.0, 1.0, 1.0], [5.5, 4.0, 6.0]]),
                          [3.0, 3.0], width=0.9)
    rho[0, 0, 0] = -1e-5
    rho[1, 2, 3] = 0.0
    assert np.array_equal(rho, golden["B_rho"])


OPT_METHODS = ("CG-PR", "CG-DY", "CG-CD", "CG-LS", "CG-FR", "GD", "DIIS")


@pytest.fixture(scope="module")
def golden_opt():
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_opt.npz")))


@pytest.mark.parametrize("method", OPT_METHODS)
def test_optimizer_methods_short(golden, golden_opt, method):
    """The oracle's CG betas, GD and DIIS against the reference's own runs
    (tests/golden/make_golden_opt.py): 10 iterations (DIIS: 4) from the uniform
    density on the 4-atom Al cell at 32^3."""
    g, go = golden, golden_opt
    from dftpy_gb300.synthetic import fcc_cell
    lat, pos = fcc_cell(7.60)
    grid = O.Grid(lat, (32, 32, 32))
    pp = O.LocalPseudo(grid, pos, np.zeros(4, dtype=int), [(g["recpot_gp"], g["recpot_vp"])], PME=True)
    ew = O.Ewald(grid, pos, np.full(4, 3.0), PME=True)
    tot = O.Total(grid, O.make_terms(grid, "TFVW", pseudo=pp), ewald_energy=ew.energy())
    rho0 = np.full((32, 32, 32), 12.0 / grid.volume)
    key = method.replace("-", "") + "_short_"
    rho, info = O.optimize(tot, rho0, grid, method=method, maxiter=int(go[key + "maxiter"]), maxfun=50,
                           econv=1e-11 * 4)
    assert info["converged"] == int(go[key + "converged"])
    assert info["niter"] == int(go[key + "niter"])
    # an unconverged 10-step path amplifies the summation-order rounding of each
    # step (numpy's sum here, einsum in the reference) to ~1e-10: 1e-9 relative
    _close(tot(rho, ("E",))["E"], go[key + "E"], rtol=1e-9, atol=0)
    _close(info["mu"], go[key + "mu"], rtol=1e-8, atol=0)
    _close(rho.sum() * grid.dV, go[key + "N"], rtol=1e-12, atol=0)
