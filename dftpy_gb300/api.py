"""Callers of the hot path: the ASE-style calculator (src/dftpy/api/api4ase.py:11-119)
and evaluator2results (src/dftpy/interface.py:245-317), on the device backend.

``DFTpyCalculator`` follows the reference calculator's evaluator path
(``run_normal``, api4ase.py:74-107): on every change of the atoms it moves the
ions of the local pseudopotential, re-optimises the density starting from the
previous one and evaluates energy, forces and stress.  The density stays a
device field between steps, so an MD or relaxation loop moves only positions,
energies, forces and stresses between host and device.

ASE itself is not a dependency: ``atoms`` is any object with
``get_positions()`` and ``get_cell()`` in Angstrom and ``get_chemical_symbols()``
(an ``ase.Atoms`` qualifies).  The reference's INI/config driver path
(``run_config``) is not on the accelerated path.
"""
import numpy as np
import torch

from .constants import ENERGY_CONV, FORCE_CONV, STRESS_CONV
from .field import DirectField
from .grid import DirectGrid
from .ions import Ions
from .optimization import Optimization

__all__ = ["DFTpyCalculator", "evaluator2results", "all_changes"]

all_changes = ["positions", "numbers", "cell", "pbc", "initial_charges", "initial_magmoms"]


def evaluator2results(evaluator, rho=None, calcType={"E", "F"}, ions=None, split=True, **kwargs):
    """interface.py:245-317: energies (and potentials), forces and stress of a
    total functional on rho, as the dict the reference returns.  The reference
    also prints a summary; this returns the same values silently."""
    calcType = set(calcType)
    forces, stress = {}, {}
    from .functional.functional_output import FunctionalOutput
    energypotential = {"TOTAL": FunctionalOutput(name="TOTAL", energy=0.0)}
    ev_calc = calcType & {"E", "V"}
    if ev_calc:
        energypotential = evaluator.get_energy_potential(rho, calcType=ev_calc, split=split)
        if not split:
            energypotential = {"TOTAL": energypotential}
    if "F" in calcType:
        forces = evaluator.get_forces(rho, split=split)
        if not split:
            forces = {"TOTAL": forces}
    if "S" in calcType:
        stress = evaluator.get_stress(rho, split=split)
        if not split:
            stress = {"TOTAL": stress}
    results = {"density": rho, "energypotential": energypotential, "forces": forces, "stress": stress,
               "evaluator": evaluator}
    if hasattr(evaluator, "PSEUDO"):
        results["pseudo"] = evaluator.PSEUDO
    return results


def _atoms_state(atoms):
    return (np.array(atoms.get_positions(), dtype=np.float64), np.array(atoms.get_cell(), dtype=np.float64),
            tuple(atoms.get_chemical_symbols()))


def ions_from_atoms(atoms):
    """Ions.from_ase: Angstrom positions and cell converted to Bohr."""
    pos, cell, sym = _atoms_state(atoms)
    return Ions(symbols=list(sym), positions=pos, cell=cell, units="ase")


class DFTpyCalculator:
    """DFTpyCalculator(evaluator=TotalFunctional, rho=initial DirectField,
    optimizer=None, zero_stress=False): energy (eV), forces (eV/A) and stress
    (Voigt xx yy zz yz xz xy, eV/A^3) of an atoms object, as api4ase.py:11-119."""

    implemented_properties = ["energy", "forces", "stress"]

    def __init__(self, config=None, mp=None, optimizer=None, evaluator=None, rho=None, zero_stress=False, **kwargs):
        if config is not None:
            raise NotImplementedError("the INI/config driver (run_config) is not on the accelerated path; "
                                      "pass evaluator= and rho=")
        self.config = config
        self.mp = mp
        self.optimizer = optimizer
        self.evaluator = evaluator
        self.zero_stress = zero_stress
        self.dftpy_results = {"density": rho}
        self.results = {}
        self.atoms = None
        self._state = None
        self.nsteps = 0  # density optimisations run

    # ---------------------------------------------------- ASE Calculator API
    def check_state(self, atoms):
        """The changes since the last calculation (ase Calculator.check_state)."""
        if self._state is None:
            return list(all_changes)
        pos, cell, sym = _atoms_state(atoms)
        p0, c0, s0 = self._state
        changes = []
        if sym != s0:
            changes.append("numbers")
        if pos.shape != p0.shape or not np.array_equal(pos, p0):
            changes.append("positions")
        if not np.array_equal(cell, c0):
            changes.append("cell")
        return changes

    def calculate(self, atoms=None, properties=["energy"], system_changes=all_changes):
        if atoms is not None:
            self.atoms = atoms
        if self.atoms is None:
            raise ValueError("no atoms to calculate")
        if self._state is not None and system_changes is all_changes:
            system_changes = self.check_state(self.atoms)
        if len(system_changes) > 0:
            self.run(system_changes, properties=properties)
            self._state = _atoms_state(self.atoms)
            self.results = {}
        res = self.dftpy_results
        self.energy = res["energypotential"]["TOTAL"].energy * ENERGY_CONV["Hartree"]["eV"]
        self.results["energy"] = self.energy
        if "forces" in properties:
            if "TOTAL" not in res["forces"]:
                self.calc_forces()
            self.forces = res["forces"]["TOTAL"] * FORCE_CONV["Ha/Bohr"]["eV/A"]
            self.results["forces"] = self.forces
        if "stress" in properties:
            voigt = np.zeros(6)
            if not self.zero_stress:
                if "TOTAL" not in res["stress"]:
                    self.calc_stress()
                S = res["stress"]["TOTAL"]
                voigt[:3] = [S[0, 0], S[1, 1], S[2, 2]]
                voigt[3], voigt[4], voigt[5] = S[1, 2], S[0, 2], S[0, 1]
            self.stress = voigt * STRESS_CONV["Ha/Bohr3"]["eV/A3"]
            self.results["stress"] = self.stress

    def get_potential_energy(self, atoms=None, force_consistent=False):
        return self._get("energy", atoms)

    def get_forces(self, atoms=None):
        return self._get("forces", atoms)

    def get_stress(self, atoms=None):
        return self._get("stress", atoms)

    def _get(self, name, atoms):
        if atoms is not None:
            self.atoms = atoms
        changes = self.check_state(self.atoms)
        if changes or name not in self.results:
            self.calculate(self.atoms, [name], changes)
        return self.results[name]

    # ------------------------------------------------------------- DFTpy part
    def run(self, system_changes=all_changes, properties=["energy"]):
        if self.evaluator is None:
            raise ValueError("!!!Error: Please give a 'config' or 'evaluator' for the calculator")
        self.run_normal(system_changes=system_changes, properties=properties)

    def run_normal(self, system_changes=all_changes, properties=["energy"], **kwargs):
        """api4ase.py:74-107: move the ions, re-optimise from the previous density."""
        rho = self.dftpy_results.get("density", None)
        ions = ions_from_atoms(self.atoms)
        if rho is None:
            raise ValueError("!!!Error: Please give a initial density for the calculator")
        grid = rho.grid
        rho_old = None
        # a new cell gets a new grid of the same shape (the reference re-grids on every
        # reported cell change; an unchanged lattice keeps the grid and its plans)
        if "cell" in system_changes and not np.allclose(ions.cell, grid.lattice, rtol=1e-12, atol=0.0):
            grid = DirectGrid(ions.cell, grid.nr)
            rho_old = rho
            rho = DirectField(grid, dtype=rho_old.dtype)
        for func in self.evaluator.funcDict.values():
            if func.type == "PSEUDO":
                func.restart(ions=ions, grid=grid)
        if rho_old is not None:
            # field2distrib on an unchanged point count is a copy; then the electron count
            rho.as_subclass(torch.Tensor).copy_(rho_old.as_subclass(torch.Tensor))
            rho = rho * (ions.get_ncharges() / float(rho.integral()))
        if self.optimizer is None:
            self.optimizer = Optimization(EnergyEvaluator=self.evaluator)
        rho = self.optimizer.optimize_rho(guess_rho=rho)
        self.nsteps += 1
        calcType = ["E"]
        if "forces" in properties:
            calcType.append("F")
        if "potential" in properties:
            calcType.append("V")
        if "stress" in properties and not self.zero_stress:
            calcType.append("S")
        self.dftpy_results = evaluator2results(self.evaluator, rho=rho, calcType=calcType, ions=ions, **kwargs)

    def calc_forces(self):
        res = self.dftpy_results
        r = evaluator2results(res.get("evaluator"), rho=res.get("density"), calcType=["F"])
        res["forces"] = r.get("forces", None)

    def calc_stress(self):
        res = self.dftpy_results
        r = evaluator2results(res.get("evaluator"), rho=res.get("density"), calcType=["S"])
        res["stress"] = r.get("stress", None)
