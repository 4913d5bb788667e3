"""The reduction entry point that allocates nothing (ofdft_dot_noalloc).

It serves callers that cannot allocate device memory where they need a
reduction: allocator and memory-pool hooks, loops that forbid allocation after
start-up, processes whose memory a framework pool has reserved.  It must give
the same float64 sum as ofdft_dot, the entry point that uses a grid handle's
allocated scratch, and keep doing so on consecutive calls that share its static
scratch.  This file is collected last so that a failure here leaves every other
test already run; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from dftpy_gb300 import _lib


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dot_handle(x, y):
    """Reference value from ofdft_dot on a grid handle of the same shape."""
    lib = _lib.load()
    nr = (C.c_int * 3)(*x.shape)
    lat = np.eye(3).ravel() * 10.0
    g = C.c_void_p()
    prec = _lib.F32 if x.dtype == torch.float32 else _lib.F64
    _lib.check(lib.ofdft_grid_create(nr, _lib.dptr(lat), prec, C.byref(g)))
    try:
        out = C.c_double()
        _lib.check(lib.ofdft_dot(g, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()) if y is not None else None,
                                 C.byref(out), _stream()))
        return out.value
    finally:
        lib.ofdft_grid_destroy(g)


def _dot_noalloc(x, y, out):
    lib = _lib.load()
    prec = _lib.F32 if x.dtype == torch.float32 else _lib.F64
    _lib.check(lib.ofdft_dot_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()) if y is not None else None,
                                     x.numel(), prec, C.c_void_p(out.data_ptr()), _stream()))
    torch.cuda.current_stream().synchronize()
    return float(out.item())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_noalloc_matches_handle_dot_twice(dtype):
    torch.cuda.set_device(0)
    gen = torch.Generator(device="cuda").manual_seed(7)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # two calls in a row, the larger first: the second uses fewer blocks, so a
    # stale partial of the first call would change its sum if it were read
    for shape in ((64, 64, 64), (37, 41, 43)):
        x = torch.randn(shape, dtype=dtype, device="cuda", generator=gen)
        y = torch.randn(shape, dtype=dtype, device="cuda", generator=gen)
        for b in (y, None):
            ref = _dot_handle(x, b)
            got = _dot_noalloc(x, b, out)
            assert abs(got - ref) <= 1e-12 * max(1.0, float((x.double().abs() * (b.double().abs() if b is not None
                                                                                    else 1.0)).sum())), (got, ref)


def test_noalloc_at_size_limit():
    """n = 67,108,864 (every one of the 4096 static partials in use), float32,
    against a float64 sum of the same values; then a small call after it."""
    torch.cuda.set_device(0)
    gen = torch.Generator(device="cuda").manual_seed(11)
    n = 67108864
    x = torch.rand(n, dtype=torch.float32, device="cuda", generator=gen)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    got = _dot_noalloc(x, None, out)
    ref = float(x.double().sum().item())
    assert abs(got - ref) <= 1e-12 * n, (got, ref)
    y = x[:1000]
    got2 = _dot_noalloc(y, None, out)
    assert abs(got2 - float(y.double().sum().item())) <= 1e-12 * 1000
    del x


def test_noalloc_rejects_oversize():
    lib = _lib.load()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    # the size check runs on the host before any launch, so no kernel touches x
    rc = lib.ofdft_dot_noalloc(C.c_void_p(x.data_ptr()), None, 67108864 + 1, _lib.F64, C.c_void_p(out.data_ptr()),
                               _stream())
    assert rc == _lib.EINVAL
    assert b"67108864" in lib.ofdft_last_error()
