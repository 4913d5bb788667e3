"""Field helpers of src/dftpy/utils/utils.py on the device: Fourier
interpolation between grids of one cell (grid_map_data) and its serial use in
field2distrib, both through ofdft_grid_map."""
import math

import torch

from . import _lib
from .field import DirectField
from .functional.abstract_functional import stream_ptr
from .grid import DirectGrid

__all__ = ["grid_map_data", "field2distrib"]


def _map(data, grid2, floor_value):
    src = data.grid
    t = data.as_subclass(torch.Tensor).contiguous()
    out = torch.empty(tuple(int(x) for x in grid2.nrR), dtype=t.dtype, device=t.device)
    _lib.check(_lib.load().ofdft_grid_map(src.native_for(t.dtype), grid2.native_for(t.dtype),
                                          _lib.C.c_void_p(t.data_ptr()), _lib.C.c_void_p(out.data_ptr()),
                                          float(floor_value), stream_ptr()))
    f = out.as_subclass(DirectField)
    f.grid = grid2
    f._N = None
    return f


def grid_map_data(data, nr=None, direct=True, index=None, grid=None):
    """utils.py:80-128: ``data`` (a DirectField) on the grid of the same cell
    with ``nr`` points (or on ``grid``); the coefficients keep their
    frequencies."""
    if not direct:
        raise NotImplementedError("grid_map_data: only the real-space result (direct=True) is supported")
    if index is not None:
        raise NotImplementedError("grid_map_data: precomputed index maps are not supported")
    if grid is None:
        grid = DirectGrid(data.grid.lattice, nr)
    elif hasattr(grid, "get_direct"):
        grid = grid.get_direct()
    return _map(data, grid, -math.inf)


def field2distrib(data, out, root=None, tol=1e-30):
    """utils.py:218-285 in one process: a copy when the grids agree, otherwise
    grid_map_data onto out's grid with values below tol raised to tol."""
    t = out.as_subclass(torch.Tensor)
    if tuple(data.grid.nrR) == tuple(out.grid.nrR):
        t.copy_(data.as_subclass(torch.Tensor))
        return out
    t.copy_(_map(data.to(t.dtype) if data.dtype != t.dtype else data, out.grid, tol).as_subclass(torch.Tensor))
    return out
