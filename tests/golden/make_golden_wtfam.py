"""Generate tests/golden/reference_wtfam.npz: the Smargiassi-Madden and Perrot
kinetic functionals (src/dftpy/functional/kedf/sm.py, fp.py: the WT engine with
their own exponents), WTE (wte.py) and the MGP kernels (mgp.py) computed by the
REFERENCE implementation, energy, potential and (but for MGP) stress, on the
smooth anisotropic density of system A.

Run in a container that has the reference sources:

    python tests/golden/make_golden_wtfam.py <reference source tree>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden import ref_objects, setup  # noqa: E402

CASES = [("SM", "SM", {}), ("FP", "FP", {}), ("SMNL", "SM-NL", {}), ("SMA", "SM", {"alpha": 0.6, "beta": 0.6}),
         ("WTE", "WTE", {}), ("WTENL", "WTE-NL", {}), ("WTEX", "WTE", {"x": 0.8, "alpha": 0.9, "beta": 0.7})]
TTF_CASES = [("TTF1", "TFVW", {"temperature": 0.5}), ("TTF2", "TF", {"temperature": 1.2, "x": 0.9}),
             ("TTF0", "TFVW", {"temperature0": 0.5}), ("TTFW", "WT", {"temperature": 0.05})]
# the density-independent MGP kernels (mgp.py): energy and potential only (no stress engine)
MGP_CASES = [("MGP", "MGP", {}), ("MGPA", "MGPA", {}), ("MGPG", "MGPG", {}), ("MGP0", "MGP0", {}),
             ("MGPNL", "MGP-NL", {"maxpoint": 200, "lumpfactor": None}),
             ("MGP0L", "MGP0", {"lumpfactor": [0.1, 0.3, 2.0]}), ("MGPS", "MGP", {"symmetrization": "Geometric"})]


def main(ref_root):
    setup(ref_root)
    DirectGrid, DirectField, Ions = ref_objects()
    from dftpy.functional.kedf import KEDF

    g0 = dict(np.load(os.path.join(HERE, "reference_golden.npz")))
    out = {}
    grid = DirectGrid(lattice=g0["A_lattice"], nr=g0["A_nr"], full=False)
    for tag, name, kw in CASES:
        f = KEDF(name=name, **kw)
        rho = DirectField(grid=grid, data=g0["A_rho"].copy())
        r = f(rho)
        out["A_E_" + tag] = float(r.energy)
        out["A_V_" + tag] = np.asarray(r.potential)
        out["A_S_" + tag] = np.asarray(f.stress(DirectField(grid=grid, data=g0["A_rho"].copy())))
        print(tag, r.energy)
    # the finite-temperature TF correction (tf.py:83-204, added by a temperature option)
    for tag, name, kw in TTF_CASES:
        rho = DirectField(grid=grid, data=g0["A_rho"].copy())
        f = KEDF(name=name, **kw)
        r = f(rho)
        out["A_E_" + tag] = float(r.energy)
        out["A_V_" + tag] = np.asarray(r.potential)
        parts = f(DirectField(grid=grid, data=g0["A_rho"].copy()), split=True)
        out["A_EDTTF_" + tag] = float(parts["DTTF"].energy)
        print(tag, r.energy, parts["DTTF"].energy)
    for tag, name, kw in MGP_CASES:
        rho = DirectField(grid=grid, data=g0["A_rho"].copy())
        r = KEDF(name=name, **kw)(rho)
        out["A_E_" + tag] = float(r.energy)
        out["A_V_" + tag] = np.asarray(r.potential)
        print(tag, r.energy)
    np.savez_compressed(os.path.join(HERE, "reference_wtfam.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
