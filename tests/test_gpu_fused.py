"""GPU checks of the fused float32 k_F-node pipeline (hand-written tile FFTs
with the node kernel, interpolation and hat weights folded in) against the
float64 path, which matches the reference to 1e-10 (test_gpu_parity.py), and
against the float32 cuFFT pipeline.

Bars, float32 against float64 on the same density: energy within 2e-6
relative; potential within 1e-5 of max|V| (float32 grids and transforms).
The cases cover every tile-FFT length the fused path instantiates (columns
32..256, rows 16..256), kdd 1, 2 and 3, linear and cubic Hermite interpolation,
node batches that accumulate into pot1/pot3/pot2 over several passes, and user
k_F bounds that put points in the small-k_F branch of the first node and clip
the largest k_F; on n1 = n2 = 256
grids the split variant (the axis-1 transform of both chains factored as
radix 8 x 32 between their column and row passes, so no axis-1 plane pass),
which must also agree with the three-pass pipeline.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn

WGC = dict(alpha=(5 + np.sqrt(5)) / 6, beta=(5 - np.sqrt(5)) / 6)
E_RTOL = 2e-6
V_RTOL = 1e-5

CASES = [
    # grid, nsp, kdd, extra options
    ((32, 32, 32), 16, 3, {}),
    ((64, 32, 64), 32, 3, {}),
    ((32, 64, 128), 16, 2, {}),
    ((64, 64, 64), 64, 1, {}),
    ((32, 32, 512), 16, 3, {}),
    ((256, 32, 32), 16, 3, {}),
    ((128, 128, 128), 64, 3, {}),
    ((64, 64, 64), 32, 3, {"max_batch": 7}),
    ((64, 64, 64), 24, 3, {"kfmin": "lift", "kfmax": "cut"}),
    # the cubic Hermite interpolation (P and M planes both feed pot1 and pot3; two hat planes per node)
    ((64, 64, 64), 32, 3, {"interp": "hermite"}),
    ((32, 64, 128), 16, 2, {"interp": "hermite"}),
    ((64, 32, 64), 24, 1, {"interp": "hermite"}),
    ((64, 64, 64), 32, 3, {"interp": "hermite", "max_batch": 7}),
    # with kdd = 3 the Hermite pot3 holds (h00' P_j + h01' P_j+1)/dk, a difference across one node
    # interval, which multiplies float32 round-off of P by |P|/|P_j+1 - P_j|: 24 nodes over the
    # narrow k_F range of lifted and cut bounds reach 1.2e-5 of max|V| in float32, so the bar is 3e-5
    ((64, 64, 64), 24, 3, {"interp": "hermite", "kfmin": "lift", "kfmax": "cut", "vtol": 3e-5}),
    ((128, 128, 128), 64, 3, {"interp": "hermite"}),
    # n1 = n2 = 256: both chains with axis 1 split between their two passes
    ((32, 256, 256), 16, 3, {}),
    ((64, 256, 256), 24, 3, {"max_batch": 7}),
    ((32, 256, 256), 12, 2, {"kfmin": "lift", "kfmax": "cut"}),
    ((32, 256, 256), 8, 1, {}),
]


def _density(nr, seed=3):
    lat = np.diag([7.6 * nr[0] / 32, 7.6 * nr[1] / 32, 7.6 * nr[2] / 32])
    rho = syn.smooth_density(lat, nr, 4.0 * np.prod(nr) / 32768, seed=seed, amp=0.4)
    return lat, rho


def _run(grid, rho, dtype, pipe, nsp, kdd, opts):
    f = D.Functional(type="KEDF", name="LWT-NL", nsp=nsp, kdd=kdd, pipeline=pipe, **WGC, **opts)
    o = f(D.DirectField(grid, data=rho, dtype=dtype))
    return o.energy, o.potential.as_subclass(torch.Tensor).double().cpu().numpy()


@pytest.mark.parametrize("nr,nsp,kdd,extra", CASES, ids=[f"{c[0]}-nsp{c[1]}-kdd{c[2]}-{len(c[3])}" for c in CASES])
def test_fused_f32_against_f64(nr, nsp, kdd, extra):
    lat, rho = _density(nr)
    grid = D.DirectGrid(lat, nr)
    opts = dict(extra)
    vtol = opts.pop("vtol", V_RTOL)
    kf = 2.0 * np.cbrt(3.0 * np.pi ** 2 * rho)
    if opts.get("kfmin") == "lift":
        # a fifth of the points fall below the first node (small-k_F branch)
        opts["kfmin"] = float(np.quantile(kf, 0.2))
    if opts.get("kfmax") == "cut":
        # a tenth of the points are clipped to the last node
        opts["kfmax"] = float(np.quantile(kf, 0.9))
    e64, v64 = _run(grid, rho, torch.float64, "cufft", nsp, kdd, opts)
    e32, v32 = _run(grid, rho, torch.float32, "fused-split" if nr[1:] == (256, 256) else "fused", nsp, kdd, opts)
    ec, vc = _run(grid, rho, torch.float32, "cufft", nsp, kdd, opts)
    vmax = float(np.abs(v64).max())
    assert abs(e32 - e64) <= E_RTOL * abs(e64), (e32, e64)
    assert float(np.abs(v32 - v64).max()) <= vtol * vmax
    # the two float32 pipelines agree with each other as closely
    assert abs(e32 - ec) <= E_RTOL * abs(e64), (e32, ec)
    assert float(np.abs(v32 - vc).max()) <= vtol * vmax


def test_fused_repeatable_bitwise():
    nr = (64, 64, 64)
    lat, rho = _density(nr, seed=5)
    grid = D.DirectGrid(lat, nr)
    a = _run(grid, rho, torch.float32, "fused", 32, 3, {})
    b = _run(grid, rho, torch.float32, "fused", 32, 3, {})
    assert a[0] == b[0]
    assert np.array_equal(a[1], b[1])


@pytest.mark.parametrize("nr,nsp,kdd", [((32, 256, 256), 16, 3), ((64, 256, 256), 64, 3)])
def test_split_axis1_matches_three_passes(nr, nsp, kdd):
    """The split chains (a radix-8 stage of axis 1 in the column passes, its
    32-point stage in the row passes) and the three-pass chains compute the
    same float32 transforms in a different order: same energy and potential to
    float32 round-off, and the split path is bitwise repeatable."""
    lat, rho = _density(nr, seed=7)
    grid = D.DirectGrid(lat, nr)
    e3, v3 = _run(grid, rho, torch.float32, "fused", nsp, kdd, {})
    es, vs = _run(grid, rho, torch.float32, "fused-split", nsp, kdd, {})
    es2, vs2 = _run(grid, rho, torch.float32, "fused-split", nsp, kdd, {})
    vmax = float(np.abs(v3).max())
    assert abs(es - e3) <= 2e-7 * abs(e3), (es, e3)
    assert float(np.abs(vs - v3).max()) <= 2e-6 * vmax
    assert es == es2 and np.array_equal(vs, vs2)
