"""Generate tests/golden/reference_kedf.npz: the LMGP family of the density-
dependent kernel (the LWT framework with MGP kernel tables, kedf/lwt.py:502-578,
kedf/kernel.py:267-322) computed by the REFERENCE implementation.

Run in a container that has the reference sources:

    python tests/golden/make_golden_kedf.py <reference source tree>

Cases:
  fixture  the reference's own Al_fde_rho.pp test density (read from
           reference_golden.npz, where make_golden.py stored it) with the
           reference's test functional KEDF 'LMGP' (TF + vW + LMGP-NL), whose
           energy the reference's test_functional.py pins at 2.9145872498710492
           (atol 1e-3);
  A        the smooth anisotropic density of system A (24x20x18): LMGP-NL,
           LMGPA-NL and LMGPG-NL with nsp = 16 (E and V), and LWT-NL with
           kerneltype 'MGP' and symmetrization 'Arithmetic';
  tables   every 101st point of the three MGP tables (neta 50000, etamax 50).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden import ref_objects, setup  # noqa: E402


def main(ref_root):
    setup(ref_root)
    DirectGrid, DirectField, Ions = ref_objects()
    from dftpy.functional import Functional
    from dftpy.functional.kedf import KEDF
    from dftpy.functional.kedf.kernel import MGPKernelTable

    g0 = dict(np.load(os.path.join(HERE, "reference_golden.npz")))
    out = {}

    grid = DirectGrid(lattice=g0["E_lattice"], nr=g0["E_nr"], full=False)
    rho = DirectField(grid=grid, data=g0["E_rho"].copy())
    o = Functional(type="KEDF", name="LMGP")(rho)
    out["fixture_E_LMGP"] = float(o.energy)
    print("fixture LMGP energy", o.energy, "(the reference test expects 2.9145872498710492, atol 1e-3)")

    gridA = DirectGrid(lattice=g0["A_lattice"], nr=g0["A_nr"], full=False)
    for tag, kw in (("LMGP", dict(name="LMGP-NL", nsp=16)), ("LMGPA", dict(name="LMGPA-NL", nsp=16)),
                    ("LMGPG", dict(name="LMGPG-NL", nsp=16)),
                    ("LWTMGPA", dict(name="LWT-NL", nsp=16, kerneltype="MGP", symmetrization="Arithmetic"))):
        rhoA = DirectField(grid=gridA, data=g0["A_rho"].copy())
        r = KEDF(**kw)(rhoA)
        out["A_E_" + tag] = float(r.energy)
        out["A_V_" + tag] = np.asarray(r.potential)
        print(tag, r.energy)

    eta = np.linspace(0, 50.0, 50000)
    for tag, sym in (("MGP", None), ("MGPA", "Arithmetic"), ("MGPG", "Geometric")):
        out["table_" + tag] = MGPKernelTable(eta, maxpoints=1000, symmetrization=sym)[::101]
    out["table_eta"] = eta[::101]
    np.savez_compressed(os.path.join(HERE, "reference_kedf.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
