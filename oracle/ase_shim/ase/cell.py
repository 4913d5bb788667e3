"""Minimal ``ase.cell.Cell`` stand-in (test infrastructure only).

Provides the members the reference's grid/ions code touches
(src/dftpy/grid.py:4, src/dftpy/ions.py:2): ``array``, ``volume``,
``lengths()``, ``scaled_positions``, ``cartesian_positions``, ``cellpar``,
indexing and array conversion.  Rows of ``array`` are the lattice vectors.
"""
import numpy as np


class Cell:
    def __init__(self, array):
        if isinstance(array, Cell):
            array = array.array
        a = np.array(array, dtype=np.float64)
        if a.shape == (3,):
            a = np.diag(a)
        if a.shape != (3, 3):
            raise ValueError("cell must be 3x3")
        self.array = a

    @classmethod
    def new(cls, cell=None):
        return cls(np.zeros((3, 3)) if cell is None else cell)

    @property
    def volume(self):
        return abs(float(np.linalg.det(self.array)))

    def lengths(self):
        return np.sqrt((self.array ** 2).sum(axis=1))

    def angles(self):
        a, b, c = self.array
        la, lb, lc = self.lengths()
        ang = lambda u, v, lu, lv: np.degrees(np.arccos(np.clip(np.dot(u, v) / (lu * lv), -1, 1)))
        return np.array([ang(b, c, lb, lc), ang(a, c, la, lc), ang(a, b, la, lb)])

    def cellpar(self):
        return np.concatenate([self.lengths(), self.angles()])

    def scaled_positions(self, positions):
        return np.linalg.solve(self.array.T, np.asarray(positions, dtype=np.float64).T).T

    def cartesian_positions(self, scaled_positions):
        return np.asarray(scaled_positions, dtype=np.float64) @ self.array

    def reciprocal(self):
        return np.linalg.inv(self.array).T

    @property
    def T(self):
        return self.array.T

    @property
    def shape(self):
        return self.array.shape

    def __array__(self, dtype=None, copy=None):
        return self.array if dtype is None else self.array.astype(dtype)

    def __getitem__(self, item):
        return self.array[item]

    def __setitem__(self, item, value):
        self.array[item] = value

    def __len__(self):
        return 3

    def __iter__(self):
        return iter(self.array)

    def copy(self):
        return Cell(self.array.copy())

    def __repr__(self):
        return "Cell(%s)" % self.array.tolist()
