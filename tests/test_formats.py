"""Density files (dftpy_gb300.formats): our readers on files the reference wrote
(tests/golden/make_golden_io.py), the reference's reading of files we wrote
(differences stored by the same script), and round trips."""
import os
import tempfile

import numpy as np
import pytest

from dftpy_gb300 import formats as F
from dftpy_gb300.ions import Ions

HERE = os.path.dirname(os.path.abspath(__file__))
IO = dict(np.load(os.path.join(HERE, "golden", "reference_io.npz")))


@pytest.mark.parametrize("ext,tol", [("xsf", 1e-9), ("pp", 1e-14)])
def test_read_reference_files(ext, tol):
    ions, data, info = F.read(os.path.join(HERE, "golden", "io", "ref_density." + ext))
    rho = IO["rho"]
    assert data.shape == rho.shape
    np.testing.assert_allclose(data, rho, rtol=0, atol=tol * np.abs(rho).max())
    np.testing.assert_allclose(ions.positions, IO["pos"], rtol=0, atol=1e-8)
    np.testing.assert_allclose(info["lattice"], IO["lattice"], rtol=0, atol=1e-8)
    assert ions.symbols == ["Al"] * 4


@pytest.mark.parametrize("ext", ["snpy", "xsf", "pp"])
def test_reference_reads_ours(ext):
    assert IO["compat_data_" + ext] <= 1e-12 * np.abs(IO["rho"]).max()
    assert IO["compat_pos_" + ext] <= 1e-12 * 10 and IO["compat_cell_" + ext] <= 1e-12 * 10


@pytest.mark.parametrize("ext", ["snpy", "xsf", "pp"])
@pytest.mark.parametrize("data_type", ["density", "potential"])
def test_round_trip(ext, data_type):
    rng = np.random.default_rng(4)
    lat = np.array([[7.1, 0.2, 0.0], [0.0, 7.9, 0.3], [0.1, 0.0, 8.3]])
    rho = rng.random((6, 5, 7)) + 0.01
    ions = Ions(symbols=["Al", "Mg", "Al"], positions=rng.random((3, 3)) * 5, cell=lat, charges=[3.0, 2.0, 3.0])
    with tempfile.TemporaryDirectory() as d:
        fn = os.path.join(d, "x." + ext)
        F.write(fn, ions=ions, data=rho, data_type=data_type)
        i2, d2, info = F.read(fn, data_type=data_type)
    np.testing.assert_allclose(d2, rho, rtol=1e-14 if ext != "snpy" else 0, atol=0)
    np.testing.assert_allclose(i2.positions, ions.positions, rtol=0, atol=1e-12)
    np.testing.assert_allclose(info["lattice"], lat, rtol=0, atol=1e-12)
    assert i2.symbols == ions.symbols


def test_unknown_format():
    with pytest.raises(AttributeError):
        F.guess_format("density.cube")
