"""GPU checks of the calculator (api4ase.py:11-119 on the device backend): its
energy, forces and stress equal a direct optimise + evaluate of the same
system; a relaxation loop re-optimises from the resident density (fewer
iterations than from the uniform density) and lowers the energy."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn
from dftpy_gb300.api import DFTpyCalculator
from dftpy_gb300.constants import BOHR, HARTREE


class Atoms:
    def __init__(self, pos, cell, sym):
        self.pos, self.cell, self.sym = np.array(pos, float), np.array(cell, float), list(sym)

    def get_positions(self):
        return self.pos.copy()

    def get_cell(self):
        return self.cell.copy()

    def get_chemical_symbols(self):
        return list(self.sym)


def _system(pos):
    lat, _ = syn.fcc_cell(7.6)
    gp, vp = syn.analytic_vloc(3.0, 1.0)
    grid = D.DirectGrid(lat, (32, 32, 32))
    ions = D.Ions(symbols=["Al"] * 4, positions=pos, cell=lat)
    pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": D.functional.RECPOT(r=gp, v=vp, zval=3)}, PME=True)
    tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="WT"),
                            XCFunctional=D.Functional(type="XC", name="LDA"),
                            HARTREE=D.Functional(type="HARTREE"), PSEUDO=pp)
    rho0 = D.DirectField(grid) + 12.0 / grid.volume
    return lat, grid, pp, tot, rho0


def _opts():
    return {"econv": 1e-9 * 4, "maxiter": 200, "maxfun": 50}


def test_calculator_matches_direct():
    lat, pos = syn.fcc_cell(7.6)
    pos = pos + np.random.default_rng(3).normal(0, 0.15, pos.shape)
    _, grid, pp, tot, rho0 = _system(pos)
    opt = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS", optimization_options=_opts())
    rho = opt.optimize_rho(guess_rho=rho0)
    e_dir = tot(rho, calcType={"E"}).energy * HARTREE
    f_dir = tot.get_forces(rho) * HARTREE / BOHR
    s_dir = tot.get_stress(rho) * HARTREE / BOHR ** 3

    _, grid2, pp2, tot2, rho02 = _system(pos)
    calc = DFTpyCalculator(evaluator=tot2, rho=rho02, optimizer=D.Optimization(
        EnergyEvaluator=tot2, optimization_method="LBFGS", optimization_options=_opts()))
    atoms = Atoms(pos * BOHR, lat * BOHR, ["Al"] * 4)
    e = calc.get_potential_energy(atoms)
    f = calc.get_forces(atoms)
    s = calc.get_stress(atoms)
    assert calc.nsteps == 1
    assert abs(e - e_dir) <= 1e-9 * abs(e_dir)
    np.testing.assert_allclose(f, f_dir, rtol=0, atol=1e-8)
    voigt = np.array([s_dir[0, 0], s_dir[1, 1], s_dir[2, 2], s_dir[1, 2], s_dir[0, 2], s_dir[0, 1]])
    np.testing.assert_allclose(s, voigt, rtol=0, atol=1e-9 * np.abs(voigt).max())


def test_relaxation_keeps_density_resident():
    lat, pos = syn.fcc_cell(7.6)
    pos = pos + np.random.default_rng(4).normal(0, 0.25, pos.shape)
    _, grid, pp, tot, rho0 = _system(pos)
    opt = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS", optimization_options=_opts())
    calc = DFTpyCalculator(evaluator=tot, rho=rho0, optimizer=opt)
    atoms = Atoms(pos * BOHR, lat * BOHR, ["Al"] * 4)
    energies, iters = [], []
    for step in range(6):
        energies.append(calc.get_potential_energy(atoms))
        f = calc.get_forces(atoms)
        iters.append(opt.result.niter)
        assert calc.dftpy_results["density"].is_cuda
        atoms.pos = atoms.pos + 0.02 * f  # steepest descent, Angstrom per eV/Angstrom
    assert calc.nsteps == 6
    assert energies[-1] < energies[0]
    assert all(b <= a + 1e-6 for a, b in zip(energies, energies[1:]))
    # later steps start from the previous ground state, not from the uniform density
    assert max(iters[2:]) < iters[0]


def test_restart_from_density_file(tmp_path):
    """A converged density written to snpy and read back restarts the optimiser
    at its ground state (formats/io.py, restart)."""
    from dftpy_gb300 import formats as F
    lat, pos = syn.fcc_cell(7.6)
    pos = pos + np.random.default_rng(5).normal(0, 0.1, pos.shape)
    _, grid, pp, tot, rho0 = _system(pos)
    opt = D.Optimization(EnergyEvaluator=tot, optimization_method="LBFGS", optimization_options=_opts())
    rho = opt.optimize_rho(guess_rho=rho0)
    fn = str(tmp_path / "rho.snpy")
    F.write_density(fn, data=rho, ions=pp.ions)
    back = F.read_density(fn)
    assert back.is_cuda and torch.equal(back.as_subclass(torch.Tensor), rho.as_subclass(torch.Tensor))
    _, grid2, pp2, tot2, _ = _system(pos)
    back2 = D.DirectField(grid2, data=back.as_subclass(torch.Tensor))
    opt2 = D.Optimization(EnergyEvaluator=tot2, optimization_method="LBFGS", optimization_options=_opts())
    opt2.optimize_rho(guess_rho=back2)
    assert opt2.result.niter <= 2
    assert abs(opt2.functional.energy - opt.functional.energy) <= 1e-8 * 4


def test_calculator_matches_reference(tmp_path):
    """The calculator against the reference's own DFTpyCalculator
    (api4ase.py:11-119; tests/golden/reference_calc.npz from
    tests/golden/make_golden_calc.py): three geometries in turn (displaced,
    displaced again from the resident density, strained cell with a carried
    density), energy in eV, forces in eV/A and Voigt stress in eV/A^3.  The
    same recpot file, functional and truncated-Newton options (econv 1e-12 Ha)
    as the reference run, so both reach the same ground-state density to the
    optimiser's convergence: energies within 1e-10 relative, forces within
    5e-6 eV/A (1e-7 Ha/Bohr), stress within 2e-7 eV/A^3 (measured: 2e-14,
    1.7e-6 and 7e-8)."""
    import os
    from oracle.ofdft_np import write_recpot
    gold = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_calc.npz")))
    torch.cuda.set_device(0)
    gp, vp = syn.analytic_vloc(3.0, 1.0)
    fn = str(tmp_path / "Al.recpot")
    write_recpot(fn, gp[-1], vp, header="analytic Z=3 rc=1")
    lat, pos = gold["s1_lattice"], gold["s1_pos"]
    grid = D.DirectGrid(lat, tuple(int(n) for n in gold["nr"]))
    ions = D.Ions(symbols=["Al"] * 4, positions=pos, cell=lat)
    pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": fn}, PME=True)
    tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="WT"),
                            XCFunctional=D.Functional(type="XC", name="LDA"),
                            HARTREE=D.Functional(type="HARTREE"), PSEUDO=pp)
    opt = D.Optimization(EnergyEvaluator=tot, optimization_method="TN",
                         optimization_options={"econv": float(gold["econv"]), "maxiter": 200, "maxfun": 50})
    calc = DFTpyCalculator(evaluator=tot, rho=D.DirectField(grid) + 12.0 / grid.volume, optimizer=opt)
    diffs = []
    for k in (1, 2, 3):
        atoms = Atoms(gold["s%d_pos" % k] * BOHR, gold["s%d_lattice" % k] * BOHR, ["Al"] * 4)
        e = calc.get_potential_energy(atoms)
        f = calc.get_forces(atoms)
        s = calc.get_stress(atoms)
        e_ref = float(gold["s%d_energy" % k])
        diffs.append((k, abs(e - e_ref) / abs(e_ref), float(np.abs(f - gold["s%d_forces" % k]).max()),
                      float(np.abs(s - gold["s%d_stress" % k]).max()),
                      abs(float(calc.dftpy_results["density"].integral()) - float(gold["s%d_N" % k]))))
    for k, de, df, ds, dn in diffs:
        assert de <= 1e-10 and df <= 5e-6 and ds <= 2e-7 and dn <= 1e-10, diffs
    assert calc.nsteps == 3
