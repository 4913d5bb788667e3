"""GPU parity of the HC and revHC kinetic kernels (kedf/hc.py) against the
reference's outputs (tests/golden/make_golden_hc.py), and of the FP32 path
against FP64.

Bars: FP64 energy within 1e-10 relative, potential within 1e-9 of max|V|;
FP32 energy within 1e-5 relative, potential within 1e-4 of max|V| (the k_F
field comes from float32 gradients)."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn

HERE = os.path.dirname(os.path.abspath(__file__))
HG = dict(np.load(os.path.join(HERE, "golden", "reference_hc.npz")))
NAMES = {"HC": "HC-NL", "REVHC": "REVHC-NL"}


def _np(f):
    return f.as_subclass(torch.Tensor).double().cpu().numpy()


@pytest.mark.parametrize("tag", ["HC", "REVHC"])
def test_hc_fp64_against_reference(golden, tag):
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    o = D.Functional(type="KEDF", name=NAMES[tag])(rho)
    e = HG["A_E_" + tag]
    assert abs(o.energy - e) <= 1e-10 * max(1.0, abs(e)), (o.energy, e)
    v = HG["A_V_" + tag]
    assert float(np.abs(_np(o.potential) - v).max()) <= 1e-9


@pytest.mark.parametrize("tag", ["HC", "REVHC"])
def test_hc_fixture(golden, tag):
    grid = D.DirectGrid(golden["E_lattice"], golden["E_nr"])
    rho = D.DirectField(grid, data=golden["E_rho"])
    e = D.Functional(type="KEDF", name=NAMES[tag])(rho, calcType={"E"}).energy
    assert abs(e - HG["E_E_" + tag]) <= 1e-10 * abs(e), (e, HG["E_E_" + tag])


@pytest.mark.parametrize("tag", ["HC", "REVHC"])
def test_hc_fp32_against_fp64(tag):
    nr = (48, 48, 48)
    lat = np.diag([11.4, 11.4, 11.4])
    rho_np = syn.smooth_density(lat, nr, 24.0, seed=8, amp=0.4)
    grid = D.DirectGrid(lat, nr)
    out = {}
    for dt in (torch.float64, torch.float32):
        o = D.Functional(type="KEDF", name=NAMES[tag])(D.DirectField(grid, data=rho_np, dtype=dt))
        out[dt] = (o.energy, _np(o.potential))
    (e64, v64), (e32, v32) = out[torch.float64], out[torch.float32]
    assert abs(e32 - e64) <= 1e-5 * abs(e64), (e32, e64)
    assert float(np.abs(v32 - v64).max()) <= 1e-4 * float(np.abs(v64).max())


def test_hc_has_no_stress(golden):
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    with pytest.raises(AttributeError):
        D.Functional(type="KEDF", name="HC").stress(rho)
