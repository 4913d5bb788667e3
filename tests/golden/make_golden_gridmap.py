"""Generate tests/golden/reference_gridmap.npz: Fourier interpolation between
grids of one cell (grid_map_data, src/dftpy/utils/utils.py:50-128) and its use
in field2distrib (utils.py:218-285, serial), computed by the REFERENCE
implementation on a seeded density of a 10x12x9 grid.

Run in a container that has the reference sources:

    python tests/golden/make_golden_gridmap.py <reference source tree>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden import ref_objects, setup  # noqa: E402

LAT = np.array([[7.0, 0.3, 0.0], [0.0, 8.0, 0.4], [0.2, 0.0, 6.5]])
NR = (10, 12, 9)
TARGETS = [(20, 24, 18), (15, 13, 11), (6, 8, 5), (10, 12, 9)]


def source_density():
    from dftpy_gb300 import synthetic as syn
    return syn.smooth_density(LAT, NR, 4.0, seed=60, amp=0.8)


def main(ref_root):
    setup(ref_root)
    DirectGrid, DirectField, Ions = ref_objects()
    from dftpy.utils.utils import field2distrib, grid_map_data
    out = {}
    rho = DirectField(grid=DirectGrid(lattice=LAT, nr=NR, full=False), data=source_density())
    for nr in TARGETS:
        tag = "x".join(str(n) for n in nr)
        out["map_" + tag] = np.asarray(grid_map_data(rho, nr))
    # field2distrib onto a finer grid, with values below the floor
    neg = DirectField(grid=rho.grid, data=np.asarray(rho) - 0.8 * float(np.asarray(rho).mean()))
    dst = DirectField(grid=DirectGrid(lattice=LAT, nr=(15, 13, 11), full=False))
    field2distrib(neg, dst, root=0)
    out["distrib_15x13x11"] = np.asarray(dst)
    np.savez_compressed(os.path.join(HERE, "reference_gridmap.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
