"""The ctypes binding that INTEGRATION.md gives a DFTpy maintainer, run as
written (only the library path is filled in).

CPU: its Config mirrors ofdft_config of include/ofdft.h member for member (names,
types, order), so ofdft_config_init accepts it; a struct of the wrong size is
refused without being written, and ofdft_eval_create refuses a config whose
struct_size is not the library's.
GPU: make_evaluator + compute on the golden 4-atom Al system (TF + vW + LDA +
Hartree + the local pseudopotential) give the reference's energy and potential.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

from dftpy_gb300 import _build, _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(REPO, "tests", "golden", "reference_golden.npz")


def header_config_fields():
    hdr = open(os.path.join(REPO, "include", "ofdft.h")).read()
    body = re.sub(r"/\*.*?\*/", "", re.search(r"typedef struct \{(.*?)\} ofdft_config;", hdr, re.S).group(1),
                  flags=re.S)
    types = {"unsigned int": C.c_uint, "int": C.c_int, "double": C.c_double}
    out = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        m = re.match(r"(unsigned int|int|double)\s+(.*)", decl)
        assert m, decl
        for name in m.group(2).split(","):
            name = name.strip()
            a = re.match(r"(\w+)\[(\d+)\]", name)
            out.append((a.group(1), types[m.group(1)] * int(a.group(2))) if a else (name, types[m.group(1)]))
    return out


def binding_namespace():
    md = open(os.path.join(REPO, "INTEGRATION.md")).read()
    block = re.search(r"```python\n(# dftpy/backends/gb300\.py.*?)```", md, re.S).group(1)
    _lib.load()  # builds the library when needed
    block = block.replace("/path/to/dftpy_gb300/libofdft.so", _build.LIB)
    ns = {}
    exec(compile(block, "INTEGRATION.md", "exec"), ns)
    return ns


def _same_type(a, b):
    if hasattr(a, "_length_") or hasattr(b, "_length_"):
        return getattr(a, "_length_", None) == getattr(b, "_length_", None) and a._type_ is b._type_
    return a is b


def test_binding_config_mirrors_header():
    ns = binding_namespace()
    fields = header_config_fields()
    for mirror in (ns["Config"], _lib.Config):
        got = mirror._fields_
        assert [n for n, _ in got] == [n for n, _ in fields]
        for (n, t), (_, u) in zip(got, fields):
            assert _same_type(t, u), n
        assert C.sizeof(mirror) == _lib.load().ofdft_config_size()


def test_config_init_refuses_wrong_size_without_writing():
    lib = _lib.load()
    size = lib.ofdft_config_size()
    buf = (C.c_ubyte * (size + 64))(*([0xAB] * (size + 64)))
    rc = lib.ofdft_config_init(C.cast(buf, C.POINTER(_lib.Config)), size - 8)
    assert rc == _lib.EINVAL and b"rebuild the binding" in lib.ofdft_last_error()
    assert all(b == 0xAB for b in buf)
    cfg = _lib.Config()
    _lib.check(lib.ofdft_config_init(C.byref(cfg), C.sizeof(cfg)))
    assert cfg.struct_size == size and cfg.lwt_neta == 50000


def test_eval_create_refuses_stale_struct_size():
    lib = _lib.load()
    cfg = _lib.Config()
    _lib.check(lib.ofdft_config_init(C.byref(cfg), C.sizeof(cfg)))
    cfg.struct_size = 200  # what a 25-member mirror without struct_size would carry
    e = C.c_void_p()
    # the size check runs before the grid handle is used, so no grid is needed here
    rc = lib.ofdft_eval_create(None, C.byref(cfg), C.byref(e))
    assert rc == _lib.EINVAL and b"struct_size" in lib.ofdft_last_error()
    assert not e.value


@pytest.mark.gpu
def test_binding_evaluates_golden_system():
    import torch
    torch.cuda.set_device(0)
    ns = binding_namespace()
    z = np.load(GOLD)

    class Grid:  # the two members of DFTpy's DirectGrid the binding reads
        nrR = tuple(int(n) for n in z["A_nr"])
        lattice = z["A_lattice"]

    vloc = z["A_V_PPPME"]  # LocalPseudo's potential is v_loc itself
    g, e = ns["make_evaluator"](Grid, 1 | 2, vloc=vloc)
    try:
        E, V = ns["compute"](e, z["A_rho"])
    finally:
        lib = _lib.load()
        lib.ofdft_eval_destroy(e)
        lib.ofdft_grid_destroy(g)
    keys = ("TF", "VW", "XC", "H", "PPPME")
    Eref = sum(float(z["A_E_" + k]) for k in keys)
    Vref = sum(z["A_V_" + k] for k in keys)
    assert abs(E - Eref) <= 1e-10 * 4 * max(1.0, abs(Eref)), (E, Eref)
    assert float(np.abs(V - Vref).max()) <= 1e-9
