"""Generate tests/golden/reference_gga.npz: GGA kinetic functionals
(src/dftpy/functional/kedf/gga.py) computed by the REFERENCE implementation.

Run in a container that has the reference sources:

    python tests/golden/make_golden_gga.py <reference source tree>

Cases: every functional of GGA_KEDF_list on the smooth anisotropic density of
system A (24x20x18; energy, potential and stress), LKT with user parameters
and with gga_remove_vw, and the reference's own test of GGA 'lc94' on its
Al_fde_rho.pp density (test_functional.py:10-21, energy 1.6821337114254904).
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
    from dftpy.functional.kedf.gga import GGA, GGA_KEDF_list

    g0 = dict(np.load(os.path.join(HERE, "reference_golden.npz")))
    out = {}
    grid = DirectGrid(lattice=g0["E_lattice"], nr=g0["E_nr"], full=False)
    rho = DirectField(grid=grid, data=g0["E_rho"].copy())
    e = Functional(type="KEDF", name="GGA", k_str="lc94")(rho).energy
    out["fixture_E_LC94"] = float(e)
    print("fixture GGA lc94", e, "(the reference test expects 1.6821337114254904)")

    gridA = DirectGrid(lattice=g0["A_lattice"], nr=g0["A_nr"], full=False)
    # GGA() looks names up upper-cased, so a mixed-case key ('PW91k') is unreachable
    names = sorted(n for n in GGA_KEDF_list if n.upper() in GGA_KEDF_list)
    out["names"] = np.array(names)
    cases = [(n, n, {}) for n in names] + [("LKT_P", "LKT", {"params": [1.1, 0.9]}),
                                          ("LKT_RVW", "LKT", {"gga_remove_vw": 1.0}),
                                          ("LKT_SIG", "LKT", {"sigma": 0.2}),
                                          ("LC94_SIG", "LC94", {"sigma": 0.35})]
    for tag, name, kw in cases:
        rA = DirectField(grid=gridA, data=g0["A_rho"].copy())
        r = GGA(rA, functional=name, calcType={"E", "V", "S"}, **kw)
        out["A_E_" + tag] = float(r.energy)
        out["A_V_" + tag] = np.asarray(r.potential)
        out["A_S_" + tag] = np.asarray(r.stress)
    # meta-GGA (Laplacian-level) functionals, energy and potential (no stress)
    from dftpy.functional.kedf.gga import MGGA_KEDF_list
    mcases = [(n, n, {}) for n in sorted(MGGA_KEDF_list)] + [("PGSL_SIG", "PGSL", {"sigma": 0.3}),
                                                             ("GE4_P", "GE4", {"params": [1.0, 0.2, 2.0]}),
                                                             ("PGSL_RVW", "PGSL", {"gga_remove_vw": 0.5})]
    out["mgga_names"] = np.array(sorted(MGGA_KEDF_list))
    for tag, name, kw in mcases:
        rA = DirectField(grid=gridA, data=g0["A_rho"].copy())
        r = Functional(type="KEDF", name="MGGA_" + name, **kw)(rA)
        out["A_E_M" + tag] = float(r.energy)
        out["A_V_M" + tag] = np.asarray(r.potential)
    # the LKT engine (lkt.py): GGA 'LKT-VW' plus vW
    for tag, kw in (("LKTE", {}), ("LKTE_P", {"params": [1.1]}), ("LKTE_S", {"sigma": 0.2, "y": 0.9})):
        rA = DirectField(grid=gridA, data=g0["A_rho"].copy())
        r = Functional(type="KEDF", name="LKT", **kw)(rA)
        out["A_E_" + tag] = float(r.energy)
        out["A_V_" + tag] = np.asarray(r.potential)
    # the vW term with Gaussian smoothing of its Laplacian (vw.py:29-53)
    for tag, kw in (("VW_SIG", {"sigma": 0.2}), ("TFVW_SIG", {"sigma": 0.35})):
        rA = DirectField(grid=gridA, data=g0["A_rho"].copy())
        r = Functional(type="KEDF", name=tag.split("_")[0], **kw)(rA)
        out["A_E_" + tag] = float(r.energy)
        out["A_V_" + tag] = np.asarray(r.potential)
    np.savez_compressed(os.path.join(HERE, "reference_gga.npz"), **out)
    print(len(cases) + 2, "cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
