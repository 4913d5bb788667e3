"""Pin the oracle's stress restatements against stress tensors the reference
itself produced (tests/golden/make_golden_stress.py)."""
import os
import tempfile

import numpy as np
import pytest

from oracle import ofdft_np as O

HERE = os.path.dirname(os.path.abspath(__file__))
WGC = dict(alpha=(5 + np.sqrt(5)) / 6, beta=(5 - np.sqrt(5)) / 6)


@pytest.fixture(scope="module")
def sg():
    return dict(np.load(os.path.join(HERE, "golden", "reference_stress.npz")))


@pytest.fixture(scope="module")
def tables(golden):
    from dftpy_gb300.synthetic import analytic_vloc
    tabs = [(golden["recpot_gp"], golden["recpot_vp"])]
    with tempfile.TemporaryDirectory() as d:
        gb, vb = analytic_vloc(2.0, 1.2)
        O.write_recpot(os.path.join(d, "b.recpot"), gb[-1], vb)
        gpb, vpb, _ = O.read_recpot(os.path.join(d, "b.recpot"))
    tabs.append((gpb, vpb))
    return tabs


def _close(a, ref, rel=1e-10):
    scale = max(1e-12, float(np.abs(ref).max()))
    np.testing.assert_allclose(a, ref, rtol=0, atol=rel * scale)


def _energies(rho, grid):
    return {"TF": O.tf(rho, grid, calc=("E",))["E"], "XC": O.lda(rho, grid), "H": O.hartree(rho, grid, calc=("E",))["E"]}


def test_terms_system_a(sg, tables):
    grid = O.Grid(sg["A_lattice"], sg["A_nr"])
    rho, pos = sg["A_rho"], sg["A_pos"]
    e = _energies(rho, grid)
    _close(O.tf_stress(grid, e["TF"]), sg["A_S_TF"])
    _close(O.vw_stress(rho, grid), sg["A_S_VW"])
    for key, kw in (("A_S_WT", {}), ("A_S_WTG", WGC)):
        ewt = O.WT(**kw)(rho, grid, calc=("E",))["E"]
        _close(O.wt_stress(rho, grid, ewt, **kw), sg[key])
    _close(O.lda_stress(rho, grid, e["XC"]["E"], e["XC"]["V"]), sg["A_S_XC"])
    _close(O.hartree_stress(rho, grid, e["H"]), sg["A_S_H"])
    sp = np.zeros(len(pos), dtype=int)
    for key, pme in (("A_S_PPPME", True), ("A_S_PPEX", False)):
        _close(O.pp_stress(O.LocalPseudo(grid, pos, sp, tables[:1], PME=pme), rho), sg[key])
    q = np.full(len(pos), 3.0)
    for key, pme in (("A_S_EWPME", True), ("A_S_EWEX", False)):
        _close(O.ewald_stress(O.Ewald(grid, pos, q, PME=pme)), sg[key])


def test_total_system_a(sg, tables):
    """TotalFunctional.get_stress(split=True): the per-term keys and their sum."""
    grid = O.Grid(sg["A_lattice"], sg["A_nr"])
    rho, pos = sg["A_rho"], sg["A_pos"]
    sp = np.zeros(len(pos), dtype=int)
    e = _energies(rho, grid)
    ewt = O.WT()(rho, grid, calc=("E",))["E"]
    parts = {"KEDF-TF": O.tf_stress(grid, e["TF"]), "KEDF-VW": O.vw_stress(rho, grid),
             "KEDF-NL": O.wt_stress(rho, grid, ewt), "XC": O.lda_stress(rho, grid, e["XC"]["E"], e["XC"]["V"]),
             "HARTREE": O.hartree_stress(rho, grid, e["H"]),
             "PSEUDO": O.pp_stress(O.LocalPseudo(grid, pos, sp, tables[:1], PME=True), rho),
             "II": O.ewald_stress(O.Ewald(grid, pos, np.full(len(pos), 3.0), PME=True))}
    for k, v in parts.items():
        _close(v, sg["A_T_" + k])
    _close(sum(parts.values()), sg["A_T_TOTAL"])


def test_two_species_system_b(sg, tables):
    grid = O.Grid(sg["B_lattice"], sg["B_nr"])
    rho, pos, q = sg["B_rho"], sg["B_pos"], sg["B_charges"]
    sp = np.where(q == 3.0, 0, 1)
    for key, pme in (("B_S_PPPME", True), ("B_S_PPEX", False)):
        _close(O.pp_stress(O.LocalPseudo(grid, pos, sp, tables, PME=pme), rho), sg[key])
    for key, pme in (("B_S_EWPME", True), ("B_S_EWEX", False)):
        _close(O.ewald_stress(O.Ewald(grid, pos, q, PME=pme)), sg[key])
    _close(O.vw_stress(rho, grid), sg["B_S_VW"])
    ewt = O.WT(**WGC)(rho, grid, calc=("E",))["E"]
    _close(O.wt_stress(rho, grid, ewt, **WGC), sg["B_S_WTG"])
    _close(O.hartree_stress(rho, grid, O.hartree(rho, grid, calc=("E",))["E"]), sg["B_S_H"])


def test_reference_has_no_lwt_stress(sg):
    assert int(sg["A_LWT_raises"]) == 1
