"""Local pseudopotential (src/dftpy/functional/pseudo/__init__.py:74-452,
:505-571) and the CASTEP recpot reader/writer (pseudo/recpot.py:11-62)."""
import os

import numpy as np
import torch

from .. import _lib
from ..constants import BOHR, HARTREE
from ..field import DirectField
from ..ions import as_ions
from .abstract_functional import NativeFunctional, stream_ptr

__all__ = ["LocalPseudo", "ReadPseudo", "RECPOT", "read_recpot", "write_recpot"]


def read_recpot(fname):
    """RECPOT.read (recpot.py:11-42): returns (gp [Bohr^-1], vp [Ha Bohr^3], zval).
    Values after 'END COMMENT' + 2 lines; the line before them is gmax (A^-1);
    the table ends at a line '1000' (or a single character)."""
    with open(fname) as f:
        lines = f.readlines()
    ibegin, iend = 0, None
    for i, line in enumerate(lines):
        if "END COMMENT" in line:
            ibegin = i + 3
        elif ibegin > 1 and (line.strip() == "1000" or len(line.strip()) == 1):
            iend = i
            break
    if iend is None:
        raise AttributeError("Error : Check the PP file : {}".format(fname))
    vals = " ".join(l.strip() for l in lines[ibegin:iend]).split()
    gmax = float(lines[ibegin - 1].strip()) * BOHR
    v = np.array(vals, dtype=np.float64) / HARTREE / BOHR ** 3
    r = np.linspace(0, gmax, num=len(v))
    zval = round((v[0] - v[1]) * (r[1] ** 2) / (4.0 * np.pi))
    return r, v, zval


def write_recpot(fname, gmax, v, header="dftpy_gb300"):
    """Write a recpot file: v in Ha*Bohr^3 on a uniform grid [0, gmax] (Bohr^-1)."""
    vv = np.asarray(v, dtype=np.float64) * HARTREE * BOHR ** 3
    lines = ["START COMMENT", header, "END COMMENT", "3     5", repr(float(gmax) / BOHR)]
    for i in range(0, len(vv), 3):
        lines.append("  ".join("%.17e" % x for x in vv[i:i + 3]))
    lines.append("1000")
    with open(fname, "w") as f:
        f.write("\n".join(lines) + "\n")


class RECPOT:
    """recpot engine with the reference's BasePseudo accessors."""

    def __init__(self, fname=None, r=None, v=None, zval=None):
        if fname is not None:
            r, v, zval = read_recpot(fname)
        self.r, self.v, self._zval = np.asarray(r, dtype=np.float64), np.asarray(v, dtype=np.float64), zval
        self.fname = fname

    @property
    def zval(self):
        return self._zval

    @property
    def radial_grid(self):
        return self.r

    @property
    def local_potential(self):
        return self.v

    @property
    def direct(self):
        return False


class ReadPseudo:
    """ReadPseudo (pseudo/__init__.py:630-706) for reciprocal-space tables."""

    def __init__(self, PP_list=None, **kwargs):
        if isinstance(PP_list, (list, tuple)):
            import re
            d = {}
            for item in PP_list:
                k = re.split(r"[._@-]", os.path.basename(str(item)))[0]
                d[k.capitalize()] = item
            PP_list = d
        self.PP_list = dict(PP_list)
        self._gp, self._vp, self._zval = {}, {}, {}
        for key, src in self.PP_list.items():
            if isinstance(src, (str, os.PathLike)):
                fname = str(src)
                if not os.path.isfile(fname):
                    raise FileNotFoundError("'{}' PP file for atom type {} not found".format(fname, key))
                if os.path.splitext(fname)[1].lower() != ".recpot":
                    raise NotImplementedError("only .recpot pseudopotentials are on the accelerated path")
                eng = RECPOT(fname)
            else:
                eng = src
            if getattr(eng, "direct", False):
                raise NotImplementedError("real-space pseudopotential tables are not supported")
            gp = np.asarray(getattr(eng, "radial_grid", getattr(eng, "r", None)), dtype=np.float64)
            vp = np.asarray(getattr(eng, "local_potential", getattr(eng, "v", None)), dtype=np.float64)
            self._gp[key], self._vp[key], self._zval[key] = gp, vp, eng.zval

    @property
    def gp(self):
        return self._gp

    @property
    def vp(self):
        return self._vp

    @property
    def zval(self):
        return self._zval


class LocalPseudo(NativeFunctional):
    """LocalPseudo(grid, ions, PP_list, PME=True, BsplineOrder=10)."""

    energy_slot = _lib.E_TOTAL
    out_name = "eN"

    def __init__(self, grid=None, ions=None, PP_list=None, PME=True, readpp=None, BsplineOrder=10, **kwargs):
        self.type = "PSEUDO"
        self.name = "PSEUDO"
        if readpp is not None:
            self.readpp = readpp
        elif PP_list is not None:
            self.readpp = ReadPseudo(PP_list)
        else:
            raise AttributeError("Must specify PP_list for Pseudopotentials")
        self.PME = PME
        self.BsplineOrder = BsplineOrder
        self.restart(grid, ions)

    # ------------------------------------------------------------- state
    def restart(self, grid=None, ions=None, full=False, duplicate=False):
        if duplicate:
            return self.__class__(grid=grid, ions=ions, readpp=self.readpp, PME=self.PME,
                                  BsplineOrder=self.BsplineOrder)
        self._native = {}
        self._vreal = {}
        self._version = object()
        self.ewald = None
        self._ions = None
        self._grid = None
        if ions is not None:
            self.ions = ions
        if grid is not None:
            self.grid = grid

    @property
    def grid(self):
        if self._grid is None:
            raise AttributeError("Must specify grid for Pseudopotentials")
        return self._grid

    @grid.setter
    def grid(self, value):
        self._grid = value.get_direct() if hasattr(value, "get_direct") else value
        self._native, self._vreal, self._version = {}, {}, object()

    @property
    def ions(self):
        if self._ions is None:
            raise AttributeError("Must specify ions for Pseudopotentials")
        return self._ions

    @ions.setter
    def ions(self, value):
        ions = as_ions(value)
        for key in ions.symbols_uniq:
            if key not in self.readpp.PP_list:
                raise ValueError("There is no pseudopotential for {:4s} atom".format(key))
        ions.set_charges(self.zval)
        if value is not ions and hasattr(value, "set_charges"):
            try:
                value.set_charges(self.zval)
            except Exception:
                pass
        self._ions = ions
        self._native, self._vreal, self._version = {}, {}, object()

    @property
    def zval(self):
        return self.readpp.zval

    @property
    def PP_list(self):
        return self.readpp.PP_list

    @property
    def species_keys(self):
        return sorted(self.readpp.PP_list)

    def _handle(self, dtype):
        h = self._native.get(dtype)
        if h is None:
            lib = _lib.load()
            keys = self.species_keys
            gps = [np.ascontiguousarray(self.readpp.gp[k]) for k in keys]
            vps = [np.ascontiguousarray(self.readpp.vp[k]) for k in keys]
            npts = (_lib.C.c_int * len(keys))(*[len(g) for g in gps])
            gpp = (_lib._PD * len(keys))(*[_lib.dptr(g) for g in gps])
            vpp = (_lib._PD * len(keys))(*[_lib.dptr(v) for v in vps])
            ptr = _lib.C.c_void_p()
            _lib.check(lib.ofdft_pseudo_create(self.grid.native_for(dtype), len(keys), npts, gpp, vpp,
                                               1 if self.PME else 0, int(self.BsplineOrder), _lib.C.byref(ptr)))
            ions = self.ions
            pos = np.ascontiguousarray(ions.positions, dtype=np.float64)
            spec = np.ascontiguousarray([keys.index(s) for s in ions.symbols], dtype=np.int32)
            rc = lib.ofdft_pseudo_set_ions(ptr, ions.nat, _lib.dptr(pos), spec.ctypes.data_as(_lib._PI))
            if rc != _lib.OK:
                lib.ofdft_pseudo_destroy(ptr)
                _lib.check(rc)
            h = _PseudoHandle(lib, ptr, (gps, vps))
            self._native[dtype] = h
        return h.ptr

    def vreal_for(self, dtype=torch.float64):
        """v_loc on the real-space grid (local_PP, :237-246), cached per precision."""
        v = self._vreal.get(dtype)
        if v is None:
            h = self._handle(dtype)
            v = DirectField(self.grid, dtype=dtype)
            t = v.as_subclass(torch.Tensor)
            _lib.check(_lib.load().ofdft_pseudo_vloc(h, _lib.C.c_void_p(t.data_ptr()), stream_ptr()))
            self._vreal[dtype] = v
        return v

    @property
    def vreal(self):
        return self.vreal_for(torch.float64)

    def local_PP(self):
        self.vreal_for(torch.float64)

    # -------------------------------------------------------- functional
    def configure(self, cfg):
        cfg.pseudo = 1

    def prepare(self, ev, grid, dtype):
        if grid is not self.grid and not (grid == self.grid):
            raise ValueError("density grid differs from the pseudopotential grid")
        ev.set_vloc(self.vreal_for(dtype), token=(self._version, dtype))

    def forces(self, rho):
        """LocalPseudo.forces (:260-270): PME or exact structure factor."""
        if not isinstance(rho, DirectField):
            raise TypeError("rho must be DirectField")
        h = self._handle(rho.dtype)
        F = np.zeros((self.ions.nat, 3))
        t = rho.as_subclass(torch.Tensor).contiguous()
        _lib.check(_lib.load().ofdft_pseudo_forces(h, _lib.C.c_void_p(t.data_ptr()), _lib.dptr(F), stream_ptr()))
        return F

    def stress(self, rho, energy=None):
        """LocalPseudo.stress (:248-258): _StressPME (:573-611) or _Stress (:479-503);
        energy None: E_PP = int v_loc rho dV of this density."""
        if rho is None:
            raise AttributeError("Must specify rho")
        if not isinstance(rho, DirectField):
            raise TypeError("rho must be DirectField")
        h = self._handle(rho.dtype)
        S = np.zeros((3, 3))
        t = rho.as_subclass(torch.Tensor).contiguous()
        _lib.check(_lib.load().ofdft_pseudo_stress(h, _lib.C.c_void_p(t.data_ptr()),
                                                   float("nan") if energy is None else float(energy), _lib.dptr(S),
                                                   stream_ptr()))
        return S

    def vloc_grad(self, rho):
        """dE_PP/dvp: gradient of int v_loc rho dV with respect to every value of
        each species' radial table (keys as PP_list), from the device adjoint."""
        if not isinstance(rho, DirectField):
            raise TypeError("rho must be DirectField")
        h = self._handle(rho.dtype)
        keys = self.species_keys
        sizes = [len(self.readpp.gp[k]) for k in keys]
        G = np.zeros(sum(sizes))
        t = rho.as_subclass(torch.Tensor).contiguous()
        _lib.check(_lib.load().ofdft_pseudo_vloc_grad(h, _lib.C.c_void_p(t.data_ptr()), _lib.dptr(G), stream_ptr()))
        out, off = {}, 0
        for k, n in zip(keys, sizes):
            out[k] = G[off:off + n].copy()
            off += n
        return out

    def set_tables(self, tables):
        """Replace the radial tables {symbol: vp} (same grids); drops cached v_loc."""
        for k, v in tables.items():
            v = np.asarray(v, dtype=np.float64)
            if v.shape != self.readpp.vp[k].shape:
                raise ValueError("table of %s must keep its %d points" % (k, len(self.readpp.vp[k])))
            self.readpp._vp[k] = v.copy()
        self._native, self._vreal, self._version = {}, {}, object()

    def set_positions(self, positions):
        """Move the ions (Bohr); drops cached v_loc and the Ewald object."""
        self._ions.positions = np.array(positions, dtype=np.float64).reshape(self._ions.nat, 3)
        self._native, self._vreal, self._version = {}, {}, object()
        self.ewald = None

    def get_ewald(self, PME=None):
        if self.ewald is None:
            from ..ewald import ewald
            if PME is None:
                PME = self.PME
            self.ewald = ewald(ions=self.ions, grid=self.grid, PME=PME, BsplineOrder=self.BsplineOrder)
        return self.ewald


class _PseudoHandle:
    def __init__(self, lib, ptr, keep):
        self.lib, self.ptr, self.keep = lib, ptr, keep

    def __del__(self):
        try:
            if self.ptr:
                self.lib.ofdft_pseudo_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass
