"""Generate tests/golden/reference_calc.npz: the REFERENCE's ASE calculator
(src/dftpy/api/api4ase.py:11-119, Quantum-MultiScale/DFTpy) driven through a
relaxation-like sequence of geometries, on seeded inputs.

Run in a container that has the reference sources:

    python tests/golden/make_golden_calc.py <reference source tree>

The reference needs ASE, which is not installed here; oracle/ase_shim provides
the members it uses (ase.Atoms, ase.units, ase.cell, ase.calculators.calculator).
Tests read only the .npz this script writes.

System: fcc Al, 4 atoms, a = 7.6 Bohr, 32^3 grid, WT + LDA + Hartree + local
PP (PME, the analytic Z=3 rc=1.0 potential written as a recpot), truncated
Newton with econv 1e-12 Ha (tight, so that the ground-state densities and
hence the forces are pinned, not only the energies), starting from the
uniform density.  The calculator is given
the evaluator, the initial density and the optimiser (run_normal) and is
asked, for each of three geometries in turn, for the energy (eV), forces
(eV/A) and Voigt stress (eV/A^3):
  1  seeded displacements (sigma 0.15 Bohr);
  2  a second set of displacements: the density is re-optimised from the
     previous one;
  3  the cell strained (x 1.01, y 0.995, z 1.0) with fractional positions
     kept: a new grid of the same shape, the previous density carried over
     (field2distrib) and rescaled to the electron count, then re-optimised.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden import make_ions, ref_objects, setup, write_pp  # noqa: E402

ECONV = 1e-12
NR = (32, 32, 32)
STRAIN = (1.01, 0.995, 1.0)


def geometries():
    """(lattice Bohr, positions Bohr) of the three steps."""
    from dftpy_gb300 import synthetic as syn
    lat, pos0 = syn.fcc_cell(7.6)
    rng = np.random.default_rng(21)
    p1 = pos0 + rng.normal(0, 0.15, pos0.shape)
    p2 = p1 + rng.normal(0, 0.05, pos0.shape)
    lat3 = lat * np.array(STRAIN)[:, None]
    p3 = (p2 @ np.linalg.inv(lat)) @ lat3
    return [(lat, p1), (lat, p2), (lat3, p3)]


def main(ref_root):
    setup(ref_root)
    DirectGrid, DirectField, Ions = ref_objects()
    from ase import Atoms
    from dftpy.api.api4ase import DFTpyCalculator
    from dftpy.constants import Units
    from dftpy.functional import Functional
    from dftpy.functional.pseudo import LocalPseudo
    from dftpy.functional.total_functional import TotalFunctional
    from dftpy.optimization import Optimization

    tmp = tempfile.mkdtemp()
    ppfile = write_pp(tmp, "Al", 3.0, 1.0)
    geos = geometries()
    lat, pos = geos[0]
    grid = DirectGrid(lattice=lat, nr=NR, full=False)
    ions = make_ions(Ions, lat, pos, ["Al"] * 4, 3.0)
    pp = LocalPseudo(grid=grid, ions=ions, PP_list={"Al": ppfile}, PME=True)
    ev = TotalFunctional(KineticEnergyFunctional=Functional(type="KEDF", name="WT"),
                         XCFunctional=Functional(type="XC", name="LDA", libxc=False),
                         HARTREE=Functional(type="HARTREE"), PSEUDO=pp)
    rho0 = DirectField(grid=grid) + 12.0 / grid.volume
    opt = Optimization(EnergyEvaluator=ev, optimization_method="TN",
                       optimization_options={"econv": ECONV, "maxiter": 200, "maxfun": 50})
    calc = DFTpyCalculator(evaluator=ev, rho=rho0, optimizer=opt)
    out = {"nr": np.array(NR), "econv": ECONV, "strain": np.array(STRAIN)}
    for k, (L, P) in enumerate(geos, start=1):
        atoms = Atoms(symbols=["Al"] * 4, positions=P * Units.Bohr, cell=L * Units.Bohr, pbc=True)
        out["s%d_lattice" % k], out["s%d_pos" % k] = L, P
        out["s%d_energy" % k] = float(calc.get_potential_energy(atoms))
        out["s%d_forces" % k] = np.array(calc.get_forces(atoms))
        out["s%d_stress" % k] = np.array(calc.get_stress(atoms))
        out["s%d_mu" % k] = float(opt.mu)
        out["s%d_N" % k] = float(calc.dftpy_results["density"].integral())
        print("step", k, out["s%d_energy" % k], np.abs(out["s%d_forces" % k]).max(), out["s%d_stress" % k])
    np.savez(os.path.join(HERE, "reference_calc.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden_calc.py <reference source tree>")
    main(sys.argv[1])
