"""Generate tests/golden/reference_stress.npz: stress tensors computed by the
REFERENCE implementation (Quantum-MultiScale/DFTpy) on seeded inputs.

Run in a container that has the reference sources:

    python tests/golden/make_golden_stress.py <reference source tree>

The reference needs ASE, which is not installed here; oracle/ase_shim provides
the few members it uses.  Tests read only the .npz this script writes.

Systems:
  A  fcc Al (4 atoms, displaced), orthorhombic 7.6 Bohr cell, 24x20x18 grid:
     every term's stress (TF, vW, WT alpha = beta, WT with the WGC alpha/beta,
     LDA, Hartree, PP PME and exact, Ewald PME and exact) and
     TotalFunctional.get_stress(split=True) of WT + LDA + Hartree + PP (PME).
  B  two species (6 Al Z=3, 2 Mg Z=2) in a 7.2 x 7.9 x 8.4 Bohr cell on a
     20x24x27 grid (one odd axis): PP PME and exact, Ewald PME and exact, and
     the vW, Hartree and WT stress on an uneven density.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)

from make_golden import make_ions, ref_objects, setup, write_pp  # noqa: E402


def main(ref_root):
    setup(ref_root)
    DirectGrid, DirectField, Ions = ref_objects()
    from dftpy.ewald import ewald
    from dftpy.functional import Functional
    from dftpy.functional.kedf import KEDF
    from dftpy.functional.pseudo import LocalPseudo
    from dftpy.functional.total_functional import TotalFunctional
    from dftpy_gb300 import synthetic as syn

    tmp = tempfile.mkdtemp()
    ppA = write_pp(tmp, "Al", 3.0, 1.0)
    ppB = write_pp(tmp, "Mg", 2.0, 1.2)
    wgc = dict(alpha=(5 + np.sqrt(5)) / 6, beta=(5 - np.sqrt(5)) / 6)
    out = {}

    # ---- A --------------------------------------------------------------------
    lat, pos = syn.fcc_cell(7.6)
    pos = pos + np.random.default_rng(11).normal(0, 0.1, pos.shape)
    nr = (24, 20, 18)
    rho_arr = syn.smooth_density(lat, nr, 12.0, seed=3, amp=0.4)
    out["A_lattice"], out["A_pos"], out["A_nr"], out["A_rho"] = lat, pos, np.array(nr), rho_arr
    grid = DirectGrid(lattice=lat, nr=nr, full=False)
    ions = make_ions(Ions, lat, pos, ["Al"] * 4, 3.0)

    def rho():
        return DirectField(grid=grid, data=rho_arr.copy())

    out["A_S_TF"] = KEDF(name="TF").stress(rho())
    out["A_S_VW"] = KEDF(name="VW").stress(rho())
    out["A_S_WT"] = KEDF(name="WT-NL").stress(rho())
    out["A_S_WTG"] = KEDF(name="WT-NL", **wgc).stress(rho())
    out["A_S_XC"] = Functional(type="XC", name="LDA", libxc=False).stress(rho())
    h = Functional(type="HARTREE")
    h(rho())
    out["A_S_H"] = h.stress(rho())
    out["A_S_PPPME"] = LocalPseudo(grid=grid, ions=ions, PP_list={"Al": ppA}, PME=True).stress(rho())
    out["A_S_PPEX"] = LocalPseudo(grid=grid, ions=ions, PP_list={"Al": ppA}, PME=False).stress(rho())
    out["A_S_EWPME"] = ewald(ions=ions, grid=grid, PME=True).stress
    out["A_S_EWEX"] = ewald(ions=ions, grid=grid, PME=False).stress
    pp = LocalPseudo(grid=grid, ions=ions, PP_list={"Al": ppA}, PME=True)
    tot = TotalFunctional(KineticEnergyFunctional=Functional(type="KEDF", name="WT"),
                          XCFunctional=Functional(type="XC", name="LDA", libxc=False),
                          HARTREE=Functional(type="HARTREE"), PSEUDO=pp)
    tot(rho())
    st = tot.get_stress(rho(), split=True)
    for k, v in st.items():
        out["A_T_" + k] = np.asarray(v)
    # the reference has no stress engine for the density-dependent kernel
    try:
        KEDF(name="LWT", nsp=8).stress(rho())
        out["A_LWT_raises"] = 0
    except AttributeError:
        out["A_LWT_raises"] = 1

    # ---- B --------------------------------------------------------------------
    latB = np.diag([7.2, 7.9, 8.4])
    fr = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5],
                   [0.25, 0.25, 0.25], [0.75, 0.75, 0.25], [0.75, 0.25, 0.75], [0.25, 0.75, 0.75]])
    posB = fr @ latB + np.random.default_rng(23).normal(0, 0.12, fr.shape)
    symB = ["Al"] * 6 + ["Mg"] * 2
    nrB = (20, 24, 27)
    rhoB = syn.smooth_density(latB, nrB, 22.0, seed=9, amp=0.5)
    out["B_lattice"], out["B_pos"], out["B_nr"], out["B_rho"] = latB, posB, np.array(nrB), rhoB
    gridB = DirectGrid(lattice=latB, nr=nrB, full=False)
    ionsB = Ions(symbols=symB, positions=posB, cell=latB)
    ionsB.set_charges({"Al": 3.0, "Mg": 2.0})
    out["B_charges"] = np.array([3.0] * 6 + [2.0] * 2)

    def rB():
        return DirectField(grid=gridB, data=rhoB.copy())

    pl = {"Al": ppA, "Mg": ppB}
    out["B_S_PPPME"] = LocalPseudo(grid=gridB, ions=ionsB, PP_list=pl, PME=True).stress(rB())
    out["B_S_PPEX"] = LocalPseudo(grid=gridB, ions=ionsB, PP_list=pl, PME=False).stress(rB())
    out["B_S_EWPME"] = ewald(ions=ionsB, grid=gridB, PME=True).stress
    out["B_S_EWEX"] = ewald(ions=ionsB, grid=gridB, PME=False).stress
    out["B_S_VW"] = KEDF(name="VW").stress(rB())
    out["B_S_WTG"] = KEDF(name="WT-NL", **wgc).stress(rB())
    hB = Functional(type="HARTREE")
    hB(rB())
    out["B_S_H"] = hB.stress(rB())

    for k in sorted(out):
        v = np.asarray(out[k])
        print(k, v.shape if v.ndim else float(v))
    np.savez_compressed(os.path.join(HERE, "reference_stress.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
