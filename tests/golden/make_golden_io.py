"""Generate tests/golden/io/: density files written by the REFERENCE implementation
(src/dftpy/formats: snpy, xsf, qepp) for the reader tests, and the reference's
reading of files written by dftpy_gb300.formats (maximum differences stored in
reference_io.npz).

Run in a container that has the reference sources:

    python tests/golden/make_golden_io.py <reference source tree>
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden import make_ions, ref_objects, setup  # noqa: E402


def main(ref_root):
    setup(ref_root)
    DirectGrid, DirectField, Ions = ref_objects()
    from dftpy.formats import io as rio
    from dftpy_gb300 import formats as F
    from dftpy_gb300.ions import Ions as OurIons

    g0 = dict(np.load(os.path.join(HERE, "reference_golden.npz")))
    lat, pos, rho = g0["A_lattice"], g0["A_pos"], g0["A_rho"][:12, :10, :9].copy()
    grid = DirectGrid(lattice=lat, nr=rho.shape, full=False)
    ions = make_ions(Ions, lat, pos, ["Al"] * 4, 3.0)
    field = DirectField(grid=grid, data=rho)
    out = {"rho": rho, "lattice": lat, "pos": pos}
    d = os.path.join(HERE, "io")
    os.makedirs(d, exist_ok=True)
    # the reference's snpy writer calls numpy.lib.format._check_version, which numpy 2.x
    # no longer has, so only its xsf and qepp writers run here; its snpy reader
    # (np.load of each record) still runs and is checked below on our files
    for ext in ("xsf", "pp"):
        rio.write(os.path.join(d, "ref_density." + ext), ions=ions, data=field)
    # the reference reading our files
    our = OurIons(symbols=["Al"] * 4, positions=pos, cell=lat, charges=3.0)
    tmp = tempfile.mkdtemp()
    for ext in ("snpy", "xsf", "pp"):
        fn = os.path.join(tmp, "ours." + ext)
        F.write(fn, ions=our, data=rho, lattice=lat)
        ri, rd, _ = rio.read_all(fn)
        out["compat_data_" + ext] = float(np.abs(np.asarray(rd) - rho).max())
        out["compat_pos_" + ext] = float(np.abs(np.asarray(ri.positions) - pos).max())
        out["compat_cell_" + ext] = float(np.abs(np.asarray(ri.cell) - lat).max())
        print(ext, out["compat_data_" + ext], out["compat_pos_" + ext], out["compat_cell_" + ext])
    np.savez_compressed(os.path.join(HERE, "reference_io.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
