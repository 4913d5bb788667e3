"""Ions: positions (Bohr), cell, symbols and valence charges
(src/dftpy/ions.py:5-156, minus the ASE base class)."""
import numpy as np

__all__ = ["Ions", "as_ions"]


class Ions:
    def __init__(self, symbols=None, positions=None, cell=None, charges=None, scaled_positions=None, units="au",
                 **kwargs):
        from .constants import BOHR
        cell = np.array(cell, dtype=np.float64).reshape(3, 3)
        if positions is None and scaled_positions is not None:
            positions = np.asarray(scaled_positions, dtype=np.float64) @ cell
        positions = np.array(positions, dtype=np.float64).reshape(-1, 3)
        if units != "au":   # ASE units (Angstrom) -> Bohr
            cell = cell / BOHR
            positions = positions / BOHR
        self.cell = cell
        self.positions = positions
        if symbols is None:
            symbols = ["X"] * len(positions)
        self.symbols = [str(s) for s in symbols]
        if len(self.symbols) != len(self.positions):
            raise ValueError("symbols and positions differ in length")
        self._charges = None
        if charges is not None:
            self.set_charges(charges)

    @property
    def nat(self):
        return len(self.positions)

    def __len__(self):
        return self.nat

    @property
    def symbols_uniq(self):
        return np.sort(np.unique(self.symbols))

    def get_chemical_symbols(self):
        return list(self.symbols)

    def get_scaled_positions(self):
        fr = np.linalg.solve(self.cell.T, self.positions.T).T % 1.0
        fr[fr == 1.0] = 0.0
        return fr

    def set_charges(self, charges=None):
        """set_charges (ions.py:94-110): dict per symbol, a scalar, or per atom."""
        if isinstance(charges, dict):
            vals = []
            for s in self.symbols:
                if s not in charges:
                    raise AttributeError("%s not in the charges" % s)
                vals.append(charges[s])
            charges = vals
        elif isinstance(charges, (float, int)):
            charges = np.ones(self.nat) * charges
        self._charges = np.array(charges, dtype=np.float64).reshape(self.nat)

    @property
    def charges(self):
        if self._charges is None:
            raise AttributeError("Please call 'set_charges' before use 'charges'.")
        return self._charges

    def get_ncharges(self):
        return float(self.charges.sum())

    @property
    def zval(self):
        out = {}
        for s in self.symbols_uniq:
            out[s] = 0
        if self._charges is None:
            return out
        for k in out:
            for i, s in enumerate(self.symbols):
                if s == k:
                    out[k] = self._charges[i]
                    break
        return out


def as_ions(obj):
    """Accept our Ions or any object with positions/cell/symbols (e.g. the
    reference's Ions, already in Bohr)."""
    if isinstance(obj, Ions):
        return obj
    cell = getattr(obj, "cell")
    cell = getattr(cell, "array", cell)
    ions = Ions(symbols=list(obj.symbols), positions=np.asarray(obj.positions), cell=np.asarray(cell))
    try:
        ions.set_charges(np.asarray(obj.charges))
    except Exception:
        pass
    return ions
