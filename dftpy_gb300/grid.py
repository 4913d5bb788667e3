"""DirectGrid / ReciprocalGrid with the reference's conventions
(src/dftpy/grid.py:8-60, :291-415, :480-720), backed by a native grid handle.

Lattice rows are the lattice vectors in Bohr.  The reciprocal grid is the
half-complex grid of an R2C transform (the reference's default gfull=False).
G vectors are never stored by the native code; the ``g``/``gg``/``q``/``mask``
properties build them on the device on demand for callers that want them.
"""
import math
import threading

import numpy as np
import torch

from . import _lib

__all__ = ["DirectGrid", "ReciprocalGrid", "default_device"]


def default_device():
    if not torch.cuda.is_available():
        raise _lib.OfdftError("dftpy_gb300 needs a CUDA GPU (sm_103a); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


class _NativeGrid:
    """Owns one native ofdft_grid handle (one per precision per grid)."""

    def __init__(self, nr, lattice, precision):
        lib = _lib.load()
        self.lib = lib
        nr_c = (_lib.C.c_int * 3)(*[int(x) for x in nr])
        lat = np.ascontiguousarray(np.asarray(lattice, dtype=np.float64).reshape(9))
        h = _lib.C.c_void_p()
        _lib.check(lib.ofdft_grid_create(nr_c, _lib.dptr(lat), precision, _lib.C.byref(h)))
        self.h = h
        self.precision = precision

    def __del__(self):
        try:
            if self.h:
                self.lib.ofdft_grid_destroy(self.h)
                self.h = None
        except Exception:
            pass


class BaseGrid:
    def __init__(self, lattice, nr, origin=(0.0, 0.0, 0.0), full=False, **kwargs):
        self._lattice = np.array(lattice, dtype=np.float64).reshape(3, 3)
        if nr is None:
            raise ValueError("nr must be given")
        self._nrR = np.array(nr, dtype=np.int64).reshape(3)
        self._nnrR = int(np.prod(self._nrR))
        self._volume = abs(float(np.linalg.det(self._lattice)))
        self._dV = self._volume / self._nnrR
        self._nrG = self._nrR.copy()
        self._nrG[-1] = self._nrR[-1] // 2 + 1
        self._origin = np.asarray(origin, dtype=np.float64)
        # only the half-complex reciprocal grid is supported (reference default gfull=False)
        self._full = False
        self._requested_full = bool(full)

    @property
    def lattice(self):
        return self._lattice

    @property
    def cell(self):
        return self._lattice

    @property
    def nrR(self):
        return self._nrR

    @property
    def nr(self):
        return self._nrR

    @property
    def nnrR(self):
        return self._nnrR

    @property
    def nnr(self):
        return self._nnrR

    @property
    def nrG(self):
        return self._nrG

    @property
    def nnrG(self):
        return int(np.prod(self._nrG))

    @property
    def volume(self):
        return self._volume

    @property
    def dV(self):
        return self._dV

    @property
    def full(self):
        return self._full

    @property
    def origin(self):
        return self._origin

    @property
    def spacings(self):
        return np.sqrt((self._lattice ** 2).sum(axis=1)) / self._nrR

    def __eq__(self, other):
        return isinstance(other, BaseGrid) and np.allclose(self.lattice, other.lattice) and \
            np.array_equal(self.nrR, other.nrR)

    def __hash__(self):
        return hash((tuple(self._nrR), tuple(np.round(self._lattice.ravel(), 12))))


class DirectGrid(BaseGrid):
    """DirectGrid (src/dftpy/grid.py:291-415)."""

    def __init__(self, lattice, nr=None, origin=(0.0, 0.0, 0.0), full=False, ecut=None, **kwargs):
        super().__init__(lattice, nr, origin, full)
        self._ecut = ecut
        self._native = {}
        self._native_lock = threading.Lock()
        self.RPgrid = None

    def native(self, precision=_lib.F64):
        """Native grid handle of the given precision (created on first use)."""
        with self._native_lock:
            n = self._native.get(precision)
            if n is None:
                n = _NativeGrid(self._nrR, self._lattice, precision)
                self._native[precision] = n
            return n.h

    def native_for(self, dtype):
        return self.native(_lib.F32 if dtype == torch.float32 else _lib.F64)

    def get_reciprocal(self):
        if self.RPgrid is None:
            self.RPgrid = ReciprocalGrid(self)
        return self.RPgrid

    def get_direct(self):
        return self

    def guess_ecut(self):
        """grid.py:363-366."""
        lengths = np.sqrt((self._lattice ** 2).sum(axis=1))
        spacings = 0.5 * (lengths / self._nrR + lengths / (self._nrR - 1))
        return math.pi ** 2 / (2 * spacings.max() ** 2)

    @property
    def ecut(self):
        return self._ecut if self._ecut is not None else self.guess_ecut()


class ReciprocalGrid(BaseGrid):
    """Half-complex reciprocal grid (src/dftpy/grid.py:480-720)."""

    def __init__(self, direct):
        rl = (2.0 * np.pi * np.linalg.inv(direct.lattice)).T
        super().__init__(rl, direct.nrR, full=False)
        self.Dgrid = direct
        self._g = self._gg = None

    def get_direct(self):
        return self.Dgrid

    def get_reciprocal(self):
        return self

    def _freqs(self, device):
        n = self.nrR
        ax = [torch.tensor(np.fft.fftfreq(n[0], d=1.0 / n[0]), dtype=torch.float64, device=device),
              torch.tensor(np.fft.fftfreq(n[1], d=1.0 / n[1]), dtype=torch.float64, device=device),
              torch.tensor(np.fft.rfftfreq(n[2], d=1.0 / n[2]), dtype=torch.float64, device=device)]
        return torch.meshgrid(*ax, indexing="ij")

    @property
    def g(self):
        if self._g is None:
            dev = default_device()
            S = self._freqs(dev)
            B = torch.tensor(self.lattice, dtype=torch.float64, device=dev)
            self._g = torch.stack([S[0] * B[0, k] + S[1] * B[1, k] + S[2] * B[2, k] for k in range(3)])
        return self._g

    @property
    def gg(self):
        if self._gg is None:
            g = self.g
            self._gg = g[0] * g[0] + g[1] * g[1] + g[2] * g[2]
        return self._gg

    @property
    def q(self):
        return torch.sqrt(self.gg)

    @property
    def invgg(self):
        gg = self.gg.clone()
        gg[0, 0, 0] = 1.0
        inv = 1.0 / gg
        inv[0, 0, 0] = 0.0
        return inv

    @property
    def g2max(self):
        return 2.0 * self.Dgrid.ecut
