"""Host logic of the ASE-style calculator (dftpy_gb300.api.DFTpyCalculator,
api4ase.py:11-119) with a fake evaluator and optimiser: change detection,
one density optimisation per change of the atoms, unit conversion and Voigt
order.  No GPU is involved."""
import numpy as np
import pytest

from dftpy_gb300.api import DFTpyCalculator
from dftpy_gb300.constants import BOHR, ENERGY_CONV, FORCE_CONV, HARTREE, STRESS_CONV


class Atoms:
    def __init__(self, pos, cell, sym):
        self.pos, self.cell, self.sym = np.array(pos, float), np.array(cell, float), list(sym)

    def get_positions(self):
        return self.pos.copy()

    def get_cell(self):
        return self.cell.copy()

    def get_chemical_symbols(self):
        return list(self.sym)


class Out:
    def __init__(self, energy):
        self.energy = energy


class FakeGrid:
    def __init__(self, lattice):
        self.lattice = np.array(lattice, float)
        self.nr = np.array([8, 8, 8])


class FakeRho:
    def __init__(self, grid):
        self.grid = grid


class FakePseudo:
    type = "PSEUDO"

    def __init__(self):
        self.restarts = []

    def restart(self, ions=None, grid=None):
        self.restarts.append(ions.positions.copy())


class FakeEvaluator:
    def __init__(self):
        self.PSEUDO = FakePseudo()
        self.funcDict = {"PSEUDO": self.PSEUDO}
        self.calls = {"E": 0, "F": 0, "S": 0}

    def get_energy_potential(self, rho, calcType, split):
        self.calls["E"] += 1
        return {"TOTAL": Out(-2.5)}

    def get_forces(self, rho, split):
        self.calls["F"] += 1
        return {"TOTAL": np.arange(12, dtype=float).reshape(4, 3) * 1e-3}

    def get_stress(self, rho, split):
        self.calls["S"] += 1
        S = np.array([[1.0, 4.0, 5.0], [4.0, 2.0, 6.0], [5.0, 6.0, 3.0]]) * 1e-4
        return {"TOTAL": S}


class FakeOptimizer:
    def __init__(self):
        self.n = 0

    def optimize_rho(self, guess_rho):
        self.n += 1
        return guess_rho


@pytest.fixture
def setup():
    lat_bohr = np.eye(3) * 7.6
    atoms = Atoms(np.array([[0, 0, 0], [0, 3.8, 3.8], [3.8, 0, 3.8], [3.8, 3.8, 0]]) * BOHR, lat_bohr * BOHR,
                  ["Al"] * 4)
    ev, opt = FakeEvaluator(), FakeOptimizer()
    calc = DFTpyCalculator(evaluator=ev, optimizer=opt, rho=FakeRho(FakeGrid(lat_bohr)))
    return atoms, ev, opt, calc


def test_units_and_voigt(setup):
    atoms, ev, opt, calc = setup
    assert calc.get_potential_energy(atoms) == pytest.approx(-2.5 * HARTREE, rel=1e-15)
    F = calc.get_forces(atoms)
    np.testing.assert_allclose(F, np.arange(12).reshape(4, 3) * 1e-3 * HARTREE / BOHR, rtol=1e-15)
    s = calc.get_stress(atoms)
    np.testing.assert_allclose(s, np.array([1, 2, 3, 6, 5, 4]) * 1e-4 * HARTREE / BOHR ** 3, rtol=1e-15)
    assert ENERGY_CONV["Hartree"]["eV"] == HARTREE
    assert FORCE_CONV["Ha/Bohr"]["eV/A"] == HARTREE / BOHR
    assert STRESS_CONV["Ha/Bohr3"]["GPa"] == pytest.approx(HARTREE / BOHR ** 3 * 160.21766208, rel=1e-9)


def test_one_optimisation_per_change(setup):
    atoms, ev, opt, calc = setup
    calc.get_potential_energy(atoms)
    calc.get_forces(atoms)
    calc.get_stress(atoms)
    calc.get_potential_energy(atoms)
    assert opt.n == 1 and calc.nsteps == 1
    assert ev.calls["F"] == 1 and ev.calls["S"] == 1
    atoms.pos[1, 0] += 0.05
    calc.get_forces(atoms)
    assert opt.n == 2 and len(ev.PSEUDO.restarts) == 2
    # the pseudopotential got the moved ions, in Bohr
    np.testing.assert_allclose(ev.PSEUDO.restarts[-1][1, 0], atoms.pos[1, 0] / BOHR, rtol=1e-14)
    assert calc.check_state(atoms) == []
    atoms.cell[0, 0] *= 1.0  # unchanged
    assert calc.check_state(atoms) == []


def test_zero_stress_and_missing_inputs(setup):
    atoms, ev, opt, calc = setup
    calc.zero_stress = True
    np.testing.assert_array_equal(calc.get_stress(atoms), np.zeros(6))
    assert ev.calls["S"] == 0
    with pytest.raises(NotImplementedError):
        DFTpyCalculator(config={"JOB": {}})
    with pytest.raises(ValueError):
        DFTpyCalculator(evaluator=ev).get_potential_energy(atoms)
