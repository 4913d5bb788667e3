"""DirectField / ReciprocalField: device fields with the reference's semantics
(src/dftpy/field.py:141-430, :727-825).

Both are ``torch.Tensor`` subclasses that carry their grid, so arithmetic
stays on the device and results keep the grid attached.  ``fft()`` multiplies
by dV, ``ifft()`` divides by dV, ``integral()`` is the sum times dV, exactly as
the reference defines them; the transforms and reductions run in the native
library.  float64 tensors use the FP64 path, float32 tensors the FP32-mixed
path (FP32 storage and FFTs, float64 reductions).
"""
import numpy as np
import torch

from . import _lib
from .grid import DirectGrid, ReciprocalGrid, default_device

__all__ = ["DirectField", "ReciprocalField", "as_field"]


def _stream():
    return _lib.C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _find_grid(args, kwargs):
    for a in list(args) + list(kwargs.values()):
        if isinstance(a, (DirectField, ReciprocalField)):
            return a.grid
        if isinstance(a, (list, tuple)):
            for b in a:
                if isinstance(b, (DirectField, ReciprocalField)):
                    return b.grid
    return None


def _wrap(ret, grid):
    if grid is None:
        return ret
    if isinstance(ret, torch.Tensor) and not isinstance(ret, (DirectField, ReciprocalField)):
        dgrid = grid.get_direct() if isinstance(grid, ReciprocalGrid) else grid
        shape = tuple(ret.shape)
        if shape == tuple(int(x) for x in dgrid.nrR) and not ret.is_complex():
            out = ret.as_subclass(DirectField)
            out.grid = dgrid
            out._N = None
            return out
        if shape == tuple(int(x) for x in dgrid.nrG) and ret.is_complex():
            out = ret.as_subclass(ReciprocalField)
            out.grid = dgrid.get_reciprocal()
            return out
        return ret
    if isinstance(ret, (list, tuple)):
        return type(ret)(_wrap(r, grid) for r in ret)
    return ret


class _FieldBase(torch.Tensor):
    @classmethod
    def __torch_function__(cls, func, types, args=(), kwargs=None):
        kwargs = kwargs or {}
        grid = _find_grid(args, kwargs)
        with torch._C.DisableTorchFunctionSubclass():
            ret = func(*args, **kwargs)
            if func in (torch.Tensor.__repr__, torch.Tensor.__format__, torch.Tensor.__str__):
                return ret
            return _wrap(ret, grid)

    def numpy(self):
        return self.detach().cpu().as_subclass(torch.Tensor).numpy()

    def __array__(self, dtype=None, copy=None):
        a = self.numpy()
        return a if dtype is None else a.astype(dtype)

    def copy(self):
        return self.clone()


class DirectField(_FieldBase):
    """Real-space field on a DirectGrid (field.py:141-430)."""

    @staticmethod
    def __new__(cls, grid, memo="", rank=1, data=None, order="C", cplx=False, griddata_3d=None, griddata_C=None,
                dtype=None, device=None, **kwargs):
        if hasattr(grid, "get_direct"):
            grid = grid.get_direct()
        if not isinstance(grid, DirectGrid):
            raise TypeError("the grid argument is not an instance of DirectGrid")
        if rank != 1:
            raise NotImplementedError("only rank-1 (spin-unpolarised) fields are supported")
        if cplx:
            raise NotImplementedError("complex real-space fields are not supported")
        if data is None:
            data = griddata_3d if griddata_3d is not None else griddata_C
        shape = tuple(int(x) for x in grid.nrR)
        device = torch.device(device) if device is not None else default_device()
        if data is None:
            t = torch.zeros(shape, dtype=dtype or torch.float64, device=device)
        else:
            if isinstance(data, torch.Tensor):
                t = data.detach()
                if dtype is not None:
                    t = t.to(dtype)
                elif t.dtype not in (torch.float32, torch.float64):
                    t = t.to(torch.float64)
                t = t.to(device)
            else:
                arr = np.asarray(data)
                t = torch.as_tensor(np.ascontiguousarray(arr.reshape(shape, order=order)),
                                    dtype=dtype or torch.float64, device=device)
            t = t.reshape(shape).contiguous()
        obj = torch.Tensor._make_subclass(cls, t, False)
        obj.grid = grid
        obj.memo = memo
        obj._N = None
        return obj

    @property
    def rank(self):
        return 1

    @property
    def cplx(self):
        return False

    @property
    def N(self):
        """Electron count, cached like the reference (field.py:647-650)."""
        if getattr(self, "_N", None) is None:
            self._N = self.integral()
        return self._N

    def _native(self):
        return self.grid.native_for(self.dtype)

    def integral(self):
        """sum * dV in float64 with a fixed summation order (field.py:186-191)."""
        out = _lib.C.c_double()
        t = self.as_subclass(torch.Tensor).contiguous()
        _lib.check(_lib.load().ofdft_dot(self._native(), _lib.C.c_void_p(t.data_ptr()), None,
                                         _lib.C.byref(out), _stream()))
        return out.value * self.grid.dV

    def asum(self):
        return self.integral() / self.grid.dV

    def amean(self):
        return self.asum() / self.grid.nnrR

    def amax(self):
        return float(self.as_subclass(torch.Tensor).max())

    def amin(self):
        return float(self.as_subclass(torch.Tensor).min())

    def fft(self):
        """rfftn * dV (field.py:413-430)."""
        t = self.as_subclass(torch.Tensor).contiguous()
        cdt = torch.complex64 if t.dtype == torch.float32 else torch.complex128
        out = torch.empty(tuple(int(x) for x in self.grid.nrG), dtype=cdt, device=t.device)
        _lib.check(_lib.load().ofdft_fft(self._native(), _lib.C.c_void_p(t.data_ptr()),
                                         _lib.C.c_void_p(out.data_ptr()), _stream()))
        r = out.as_subclass(ReciprocalField)
        r.grid = self.grid.get_reciprocal()
        return r


class ReciprocalField(_FieldBase):
    """Half-complex reciprocal-space field (field.py:727-825)."""

    @staticmethod
    def __new__(cls, grid, memo="", rank=1, data=None, griddata_3d=None, dtype=None, device=None, **kwargs):
        if hasattr(grid, "get_reciprocal"):
            grid = grid.get_reciprocal()
        shape = tuple(int(x) for x in grid.nrG)
        device = torch.device(device) if device is not None else default_device()
        if data is None:
            data = griddata_3d
        if data is None:
            t = torch.zeros(shape, dtype=dtype or torch.complex128, device=device)
        elif isinstance(data, torch.Tensor):
            t = data.detach().to(device).reshape(shape).contiguous()
        else:
            t = torch.as_tensor(np.ascontiguousarray(np.asarray(data).reshape(shape)), dtype=dtype or torch.complex128,
                                device=device)
        obj = torch.Tensor._make_subclass(cls, t, False)
        obj.grid = grid
        return obj

    def ifft(self, check_real=False, force_real=True):
        """irfftn(s=nr) / dV (field.py:779-804)."""
        t = self.as_subclass(torch.Tensor).contiguous()
        dgrid = self.grid.get_direct()
        rdt = torch.float32 if t.dtype == torch.complex64 else torch.float64
        out = torch.empty(tuple(int(x) for x in dgrid.nrR), dtype=rdt, device=t.device)
        _lib.check(_lib.load().ofdft_ifft(dgrid.native_for(rdt), _lib.C.c_void_p(t.data_ptr()),
                                          _lib.C.c_void_p(out.data_ptr()), _stream()))
        r = out.as_subclass(DirectField)
        r.grid = dgrid
        r._N = None
        return r


def as_field(grid, rho, dtype=None):
    """A DirectField on ``grid`` from a DirectField, tensor or numpy array."""
    if isinstance(rho, DirectField) and (dtype is None or rho.dtype == dtype):
        return rho
    return DirectField(grid, data=rho, dtype=dtype)
