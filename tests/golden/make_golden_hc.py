"""Generate tests/golden/reference_hc.npz: the HC and revHC kinetic functionals
(src/dftpy/functional/kedf/hc.py, kernel.py:460-506) computed by the REFERENCE
implementation, energy and potential, on the smooth anisotropic density of
system A (24x20x18) and on the reference's Al_fde_rho.pp test density.

Run in a container that has the reference sources:

    python tests/golden/make_golden_hc.py <reference source tree>
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
    from dftpy.functional.kedf import KEDF

    g0 = dict(np.load(os.path.join(HERE, "reference_golden.npz")))
    out = {}
    for pre in ("A_", "E_"):
        grid = DirectGrid(lattice=g0[pre + "lattice"], nr=g0[pre + "nr"], full=False)
        for tag, name in (("HC", "HC-NL"), ("REVHC", "REVHC-NL")):
            rho = DirectField(grid=grid, data=g0[pre + "rho"].copy())
            r = KEDF(name=name)(rho)
            out[pre + "E_" + tag] = float(r.energy)
            if pre == "A_":  # the fixture's potentials would make the file large
                out[pre + "V_" + tag] = np.asarray(r.potential)
            print(pre, tag, r.energy)
    np.savez_compressed(os.path.join(HERE, "reference_hc.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
