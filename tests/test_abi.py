"""CPU tests of the C ABI: the library builds and loads, exports every entry
point include/ofdft.h declares, rejects bad arguments with a status, and its
host-side MINPACK-2 line search matches scipy's line_search_wolfe1 (the
reference's line search, src/dftpy/math_utils.py:37-52)."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

from dftpy_gb300 import _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(REPO, "include", "ofdft.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ofdft_[a-z0-9_]+)\s*\(", txt)))


def test_library_loads_and_exports_header():
    lib = _lib.load()
    syms = header_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), "missing export %s" % s
    assert set(syms) == set(_lib.exported_symbols())
    assert b"sm_103a" in lib.ofdft_version()


def test_bad_arguments_return_status():
    lib = _lib.load()
    h = C.c_void_p()
    nr = (C.c_int * 3)(1, 8, 8)
    lat = np.eye(3).ravel()
    rc = lib.ofdft_grid_create(nr, _lib.dptr(lat), _lib.F64, C.byref(h))
    assert rc == _lib.EINVAL
    assert b"grid" in lib.ofdft_last_error()
    nr = (C.c_int * 3)(8, 8, 8)
    rc = lib.ofdft_grid_create(nr, _lib.dptr(lat), 7, C.byref(h))
    assert rc == _lib.EINVAL


def test_config_defaults_match_reference():
    cfg = _lib.Config()
    _lib.load().ofdft_config_default(C.byref(cfg))
    assert cfg.lwt_ratio == 1.15 and cfg.lwt_kdd == 3 and cfg.lwt_neta == 50000 and cfg.lwt_etamax == 50.0
    assert abs(cfg.lwt_ldw - 1.0 / 6.0) < 1e-15
    assert math.isnan(cfg.lwt_kfmin) and math.isnan(cfg.lwt_kfmax)
    o = _lib.OptOptions()
    _lib.load().ofdft_opt_default(C.byref(o))
    assert (o.maxiter, o.maxfun, o.ncheck, o.maxcor) == (200, 50, 2, 6)
    assert (o.c1, o.c2, o.xtol, o.econv) == (1e-4, 0.2, 1e-12, 1e-5)
    # the options the reference lacks are off by default
    assert (o.pconv, o.ls_grad, o.ls_start) == (0.0, 0, 0)


def test_optimizer_line_search_options():
    """linesearch / linesearch_start map to ls_grad / ls_start; unknown values fail
    where the options are read (no GPU needed: the struct is filled on the host)."""
    import dftpy_gb300 as D
    tot = D.TotalFunctional()
    o = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS",
                       optimization_options={"linesearch": "grad", "linesearch_start": "direction"})
    s = o.options_struct()
    assert (s.ls_grad, s.ls_start) == (1, 1)
    s = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS").options_struct()
    assert (s.ls_grad, s.ls_start) == (0, 0)
    bad = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS",
                         optimization_options={"linesearch_start": "newton"})
    with pytest.raises(ValueError):
        bad.options_struct()


def _native_ls(f, fp, c1=1e-4, c2=0.2, amax=np.pi, amin=0.0, xtol=1e-12):
    calls = []

    def cb(a, fo, go, ctx):
        fo[0] = f(a)
        go[0] = fp(a)
        calls.append(a)
        return 0

    fn = _lib.PHI_FN(cb)
    stp, fv, gv, n = C.c_double(), C.c_double(), C.c_double(), C.c_int()
    _lib.check(_lib.load().ofdft_linesearch(fn, None, f(0.0), fp(0.0), 1.0, c1, c2, amax, amin, xtol, 100,
                                            C.byref(stp), C.byref(fv), C.byref(gv), C.byref(n)))
    return (None if math.isnan(stp.value) else stp.value), n.value, calls


CASES = [
    (lambda a: (a - 0.3) ** 2 - 1.0, lambda a: 2 * (a - 0.3)),
    (lambda a: -math.sin(a) * 3 + 0.1 * a ** 4, lambda a: -math.cos(a) * 3 + 0.4 * a ** 3),
    (lambda a: 1.0 - math.cos(2.3 * a) + 0.01 * a, lambda a: 2.3 * math.sin(2.3 * a) + 0.01 - 0.05),
    (lambda a: math.exp(-a) + 0.5 * a ** 2 - 2 * a, lambda a: -math.exp(-a) + a - 2),
    (lambda a: (a - 2.9) ** 4 - 3 * a, lambda a: 4 * (a - 2.9) ** 3 - 3),
    (lambda a: -a * 1e-3 + 1e-6 * a ** 2, lambda a: -1e-3 + 2e-6 * a),
]


@pytest.mark.parametrize("k", range(len(CASES)))
def test_linesearch_matches_scipy(k):
    from scipy.optimize._linesearch import line_search_wolfe1
    f, fp = CASES[k]
    if fp(0.0) >= 0:
        pytest.skip("not a descent direction")
    seen = []

    def ff(x):
        seen.append(float(x))
        return f(float(x))

    ref = line_search_wolfe1(ff, lambda x: fp(float(x)), 0.0, 1.0, gfk=fp(0.0), old_fval=f(0.0), c1=1e-4, c2=0.2,
                             amax=np.pi, amin=0.0, xtol=1e-12)
    stp, n, calls = _native_ls(f, fp)
    if ref[0] is None:
        assert stp is None
    else:
        assert stp is not None and abs(stp - ref[0]) <= 1e-14 * max(1.0, abs(ref[0]))
    # identical trial sequence
    assert len(calls) == len(seen)
    np.testing.assert_allclose(calls, seen, rtol=1e-14, atol=0)


def _native_grad_ls(fp, stp0, amax=np.pi / 4, c2=0.2, maxiter=20):
    lib = _lib.load()
    calls = []

    @_lib.PHI_FN
    def cb(a, f, g, ctx):
        calls.append(a)
        f[0] = 0.0
        g[0] = fp(a)
        return 0

    stp, fo, go, n = C.c_double(), C.c_double(), C.c_double(), C.c_int()
    _lib.check(lib.ofdft_linesearch_grad(cb, None, fp(0.0), stp0, c2, amax, maxiter, C.byref(stp), C.byref(fo),
                                         C.byref(go), C.byref(n)))
    return (None if np.isnan(stp.value) else stp.value), go.value, calls


@pytest.mark.parametrize("theta_min,stp0", [(0.03, 0.1), (0.5, 0.1), (0.2, 0.2), (1e-4, 0.1)])
def test_derivative_line_search_finds_the_minimum(theta_min, stp0):
    """The derivative-only search (ls_grad) on the energy along a rotation,
    E(theta) = -cos(2 (theta - theta_min)): it returns a step with
    |E'| <= 0.2 |E'(0)|, and the last trial is the accepted step."""
    fp = lambda a: 2.0 * np.sin(2.0 * (a - theta_min))
    stp, g, calls = _native_grad_ls(fp, stp0)
    assert stp is not None and calls[-1] == stp
    assert abs(g) <= 0.2 * abs(fp(0.0)) + 1e-15
    assert abs(stp - theta_min) <= 0.2 * theta_min + 1e-12


def test_derivative_line_search_refuses_bad_cases():
    # not a descent direction; still descending at the step limit (pi/4)
    assert _native_grad_ls(lambda a: 1.0 + a, 0.1)[0] is None
    assert _native_grad_ls(lambda a: 2.0 * np.sin(2.0 * (a - 1.2)), 0.1)[0] is None
