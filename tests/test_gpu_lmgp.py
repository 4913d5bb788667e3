"""GPU parity of the LMGP family (the k_F-node kernel with MGP kernel tables,
kedf/lwt.py:571-578, kedf/kernel.py:267-322) against the reference's outputs
(tests/golden/make_golden_kedf.py), and of its float32 paths against float64.

Bars: FP64 energy within 1e-10 relative, potential within 1e-9 a.u.; FP32
(fused tile-FFT pipeline on power-of-two grids, cuFFT pipeline otherwise)
energy within 2e-6 relative, potential within 1e-5 of max|V| of FP64."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = [("LMGP", dict(name="LMGP-NL")), ("LMGPA", dict(name="LMGPA-NL")), ("LMGPG", dict(name="LMGPG-NL")),
         ("LWTMGPA", dict(name="LWT-NL", kerneltype="MGP", symmetrization="Arithmetic"))]


@pytest.fixture(scope="module")
def kg():
    return dict(np.load(os.path.join(HERE, "golden", "reference_kedf.npz")))


@pytest.mark.parametrize("tag,kw", CASES, ids=[c[0] for c in CASES])
def test_lmgp_fp64_against_reference(golden, kg, tag, kw):
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    o = D.Functional(type="KEDF", nsp=16, **kw)(rho)
    e = kg["A_E_" + tag]
    assert abs(o.energy - e) <= 1e-10 * max(1.0, abs(e)), (o.energy, e)
    v = o.potential.as_subclass(torch.Tensor).cpu().numpy()
    assert float(np.abs(v - kg["A_V_" + tag]).max()) <= 1e-9


def test_lmgp_reference_fixture(golden, kg):
    """The reference's own test (test_functional.py:29-34): KEDF 'LMGP' on Al_fde_rho.pp."""
    grid = D.DirectGrid(golden["E_lattice"], golden["E_nr"])
    rho = D.DirectField(grid, data=golden["E_rho"])
    e = D.Functional(type="KEDF", name="LMGP")(rho).energy
    assert abs(e - kg["fixture_E_LMGP"]) <= 1e-10 * abs(e)
    assert np.isclose(e, 2.9145872498710492, atol=1e-3)


@pytest.mark.parametrize("nr,pipe", [((64, 64, 64), "fused"), ((48, 40, 36), "cufft")])
def test_lmgp_fp32_against_fp64(nr, pipe):
    lat = np.diag([7.6 * nr[0] / 32, 7.6 * nr[1] / 32, 7.6 * nr[2] / 32])
    rho_np = syn.smooth_density(lat, nr, 4.0 * np.prod(nr) / 32768, seed=3, amp=0.4)
    grid = D.DirectGrid(lat, nr)
    out = {}
    for dt, p in ((torch.float64, "cufft"), (torch.float32, pipe)):
        f = D.Functional(type="KEDF", name="LMGP-NL", nsp=32, pipeline=p)
        o = f(D.DirectField(grid, data=rho_np, dtype=dt))
        out[dt] = (o.energy, o.potential.as_subclass(torch.Tensor).double().cpu().numpy())
    (e64, v64), (e32, v32) = out[torch.float64], out[torch.float32]
    assert abs(e32 - e64) <= 2e-6 * abs(e64), (e32, e64)
    assert float(np.abs(v32 - v64).max()) <= 1e-5 * float(np.abs(v64).max())
