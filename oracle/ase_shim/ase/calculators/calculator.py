"""Minimal ``ase.calculators.calculator`` stand-in (test infrastructure only).

The reference's ``DFTpyCalculator`` (src/dftpy/api/api4ase.py:8-60) subclasses
``Calculator`` and imports ``all_changes``.  It uses ``Calculator.__init__``
(keyword arguments), ``Calculator.calculate`` (which stores a copy of the atoms)
and the ``results`` dict.  This module provides those, plus ``get_property``
and the ``get_potential_energy``/``get_forces``/``get_stress`` accessors with
ASE's change detection (positions, numbers, cell, pbc, initial charges),
written from ASE's documented behaviour.
"""
import numpy as np

all_changes = ["positions", "numbers", "cell", "pbc", "initial_charges", "initial_magmoms"]
all_properties = ["energy", "forces", "stress", "stresses", "dipole", "charges", "magmom", "magmoms",
                  "free_energy", "energies"]


class PropertyNotImplementedError(NotImplementedError):
    pass


def _state(atoms):
    charges = atoms.arrays.get("initial_charges")
    return {"positions": np.array(atoms.positions, dtype=np.float64),
            "numbers": tuple(atoms.get_chemical_symbols()),
            "cell": np.array(atoms.cell.array, dtype=np.float64),
            "pbc": np.array(atoms.pbc, dtype=bool),
            "initial_charges": None if charges is None else np.array(charges, dtype=np.float64)}


class Calculator:
    implemented_properties = []

    def __init__(self, restart=None, ignore_bad_restart_file=None, label=None, atoms=None, directory=".", **kwargs):
        self.atoms = None
        self.results = {}
        self.parameters = dict(kwargs)
        self.label = label
        self.directory = directory
        if atoms is not None:
            atoms.calc = self

    def check_state(self, atoms, tol=1e-15):
        if self.atoms is None:
            return list(all_changes)
        a, b = _state(self.atoms), _state(atoms)
        changes = []
        for name in ("positions", "numbers", "cell", "pbc", "initial_charges"):
            x, y = a[name], b[name]
            if x is None or y is None:
                same = x is None and y is None
            elif isinstance(x, tuple):
                same = x == y
            elif x.dtype == bool:
                same = np.array_equal(x, y)
            else:
                same = x.shape == y.shape and bool(np.all(np.abs(x - y) <= tol))
            if not same:
                changes.append(name)
        return changes

    def calculate(self, atoms=None, properties=["energy"], system_changes=all_changes):
        if atoms is not None:
            self.atoms = atoms.copy()

    def get_property(self, name, atoms=None, allow_calculation=True):
        if name not in self.implemented_properties:
            raise PropertyNotImplementedError("%s property not implemented" % name)
        if atoms is None:
            atoms = self.atoms
            changes = []
        else:
            changes = self.check_state(atoms)
            if changes:
                self.results = {}
        if name not in self.results:
            if not allow_calculation:
                return None
            self.calculate(atoms, [name], changes)
        result = self.results[name]
        return result.copy() if isinstance(result, np.ndarray) else result

    def get_potential_energy(self, atoms=None, force_consistent=False):
        return self.get_property("energy", atoms)

    def get_forces(self, atoms=None):
        return self.get_property("forces", atoms)

    def get_stress(self, atoms=None):
        return self.get_property("stress", atoms)
