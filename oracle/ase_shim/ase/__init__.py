"""Minimal ``ase`` stand-in so the reference DFTpy sources import here.

Test infrastructure only (used by the fixture generator under tests/golden/).
ASE itself is not installed in this container and cannot be.  The reference
needs ``ase.units`` (src/dftpy/constants.py:3), ``ase.cell.Cell``
(src/dftpy/grid.py:4) and ``ase.Atoms`` (src/dftpy/ions.py:2); this package
provides exactly the members those modules use, in our own code.
"""
import numpy as np

from . import units  # noqa: F401
from .cell import Cell

__all__ = ["Atoms", "Cell", "units"]


class Symbols(list):
    """List of chemical symbols; ``str(symbols)`` gives the formula string."""

    def __str__(self):
        return "".join(self)


class Atoms:
    def __init__(self, symbols=None, positions=None, numbers=None, tags=None,
                 momenta=None, masses=None, magmoms=None, charges=None,
                 scaled_positions=None, cell=None, pbc=None, celldisp=None,
                 constraint=None, calculator=None, info=None, velocities=None):
        if isinstance(symbols, Atoms):
            other = symbols
            self.cell = other.cell.copy()
            self.arrays = {k: v.copy() for k, v in other.arrays.items()}
            self._symbols = Symbols(other._symbols)
            self._celldisp = other._celldisp.copy()
            self.pbc = other.pbc.copy()
            self.info = dict(other.info)
            return
        self.cell = Cell(np.zeros((3, 3)) if cell is None else cell)
        if isinstance(symbols, str):
            symbols = _split_formula(symbols)
        if symbols is None:
            n = len(positions if positions is not None else scaled_positions)
            symbols = ["X"] * n
        self._symbols = Symbols(str(s) for s in symbols)
        n = len(self._symbols)
        if positions is None and scaled_positions is not None:
            positions = self.cell.cartesian_positions(scaled_positions)
        if positions is None:
            positions = np.zeros((n, 3))
        self.arrays = {"positions": np.array(positions, dtype=np.float64).reshape(n, 3)}
        if charges is not None:
            self.arrays["initial_charges"] = np.array(charges, dtype=np.float64)
        self._celldisp = np.zeros(3) if celldisp is None else np.array(celldisp, dtype=np.float64)
        self.pbc = np.ones(3, dtype=bool) if pbc is None else np.array(pbc, dtype=bool)
        self.info = {} if info is None else dict(info)

    # --- arrays -----------------------------------------------------------
    def has(self, name):
        return name in self.arrays

    @property
    def positions(self):
        return self.arrays["positions"]

    @positions.setter
    def positions(self, value):
        self.arrays["positions"][:] = value

    def get_positions(self):
        return self.positions.copy()

    def set_positions(self, value):
        self.positions = value

    def get_scaled_positions(self, wrap=True):
        fr = self.cell.scaled_positions(self.positions)
        if wrap:
            fr = fr % 1.0
            fr[fr == 1.0] = 0.0
        return fr

    def set_initial_charges(self, charges=None):
        if charges is None:
            self.arrays.pop("initial_charges", None)
        else:
            self.arrays["initial_charges"] = np.array(charges, dtype=np.float64).reshape(len(self))

    def get_initial_charges(self):
        return self.arrays["initial_charges"].copy()

    # --- symbols ----------------------------------------------------------
    @property
    def symbols(self):
        return self._symbols

    def get_chemical_symbols(self):
        return list(self._symbols)

    def get_cell(self):
        return self.cell

    def get_volume(self):
        return self.cell.volume

    def __len__(self):
        return len(self._symbols)

    def copy(self):
        return self.__class__(self)


def _split_formula(formula):
    out, i = [], 0
    while i < len(formula):
        j = i + 1
        while j < len(formula) and formula[j].islower():
            j += 1
        sym = formula[i:j]
        k = j
        while k < len(formula) and formula[k].isdigit():
            k += 1
        cnt = int(formula[j:k]) if k > j else 1
        out.extend([sym] * cnt)
        i = k
    return out
