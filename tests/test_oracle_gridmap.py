"""The oracle's Fourier interpolation between grids (grid_map_data,
utils/utils.py:50-128) against the reference's outputs
(tests/golden/make_golden_gridmap.py): finer, coarser, odd sizes and the same
grid; field2distrib's floor."""
import os
import sys

import numpy as np
import pytest

from oracle import ofdft_np as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden_gridmap import LAT, NR, TARGETS, source_density  # noqa: E402

GM = dict(np.load(os.path.join(HERE, "golden", "reference_gridmap.npz")))


@pytest.mark.parametrize("nr", TARGETS, ids=["x".join(map(str, t)) for t in TARGETS])
def test_grid_map(nr):
    out = O.grid_map(source_density(), O.Grid(LAT, NR), nr)
    ref = GM["map_" + "x".join(map(str, nr))]
    assert np.abs(out - ref).max() <= 1e-15


def test_field2distrib_floor():
    f = source_density()
    out = np.maximum(O.grid_map(f - 0.8 * f.mean(), O.Grid(LAT, NR), (15, 13, 11)), 1e-30)
    ref = GM["distrib_15x13x11"]
    assert (ref == 1e-30).sum() > 0
    assert np.abs(out - ref).max() <= 1e-15
