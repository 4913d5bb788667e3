"""Pin the oracle's HC / revHC restatement against the reference's outputs
(tests/golden/make_golden_hc.py)."""
import os

import numpy as np
import pytest

from oracle import ofdft_np as O

HERE = os.path.dirname(os.path.abspath(__file__))
HG = dict(np.load(os.path.join(HERE, "golden", "reference_hc.npz")))
KW = {"HC": {}, "REVHC": {"functional": "PBE2", "params": [0.1, 0.45]}}


@pytest.fixture(scope="module")
def hc_objects():
    return {tag: O.HC(**kw) for tag, kw in KW.items()}


@pytest.mark.parametrize("tag", ["HC", "REVHC"])
def test_hc_system_a(golden, hc_objects, tag):
    grid = O.Grid(golden["A_lattice"], golden["A_nr"])
    r = O.HC(**KW[tag])(golden["A_rho"], grid)
    e = HG["A_E_" + tag]
    assert abs(r["E"] - e) <= 1e-11 * max(1.0, abs(e)), (r["E"], e)
    v = HG["A_V_" + tag]
    np.testing.assert_allclose(r["V"], v, rtol=0, atol=1e-10 * np.abs(v).max())


@pytest.mark.parametrize("tag", ["HC", "REVHC"])
def test_hc_fixture(golden, tag):
    grid = O.Grid(golden["E_lattice"], golden["E_nr"])
    r = O.HC(**KW[tag])(golden["E_rho"], grid, calc=("E",))
    assert abs(r["E"] - HG["E_E_" + tag]) <= 1e-11 * abs(HG["E_E_" + tag])
