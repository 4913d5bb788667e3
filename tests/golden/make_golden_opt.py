"""Generate tests/golden/reference_opt.npz: the direction methods of the
reference's Optimization beyond TN / L-BFGS / CG-HS (CG-PR, CG-DY, CG-CD, CG-LS,
CG-FR, GD and DIIS; optimization.py:179-203, math_utils.py:326-354) on the 4-atom
fcc Al system at 32^3 (TF + vW + LDA + Hartree + PME local PP) from the uniform
density, by running the REFERENCE itself.

For each method two runs: 10 iterations (maxiter 11) and 59 iterations (maxiter
60), econv 4e-11; the reference's DIIS diverges on this system after its fourth
iteration, so it gets 4 iterations (maxiter 5) instead.  Stored per run: the
energy of the returned density, the chemical potential, the electron count, the
convergence flag and the number of iterations.

    python tests/golden/make_golden_opt.py <reference source tree>
"""
import contextlib
import io
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

METHODS = ("CG-PR", "CG-DY", "CG-CD", "CG-LS", "CG-FR", "GD", "DIIS")


def main(ref_root):
    mg.setup(ref_root)
    DirectGrid, DirectField, Ions = mg.ref_objects()
    from dftpy.functional import Functional
    from dftpy.functional.total_functional import TotalFunctional
    from dftpy.functional.pseudo import LocalPseudo
    from dftpy.optimization import Optimization
    import dftpy.optimization.optimization as OO
    from dftpy_gb300 import synthetic as syn

    tmp = tempfile.mkdtemp()
    ppA = mg.write_pp(tmp, "Al", 3.0, 1.0)
    lat1, pos1 = syn.fcc_cell(7.60)
    lines = []
    OO.sprint = lambda *a, **k: lines.append(" ".join(str(x) for x in a))
    out = {}
    for meth in METHODS:
        for tag, maxiter in (("short", 11), ("long", 60)):
            if meth == "DIIS":
                if tag == "long":
                    continue
                maxiter = 5
            lines.clear()
            grid1 = DirectGrid(lattice=lat1, nr=(32, 32, 32), full=False)
            ions1 = mg.make_ions(Ions, lat1, pos1, ["Al"] * 4, 3.0)
            PP = LocalPseudo(grid=grid1, ions=ions1, PP_list={"Al": ppA}, PME=True)
            EE = TotalFunctional(KineticEnergyFunctional=Functional(type="KEDF", name="TFVW"),
                                 XCFunctional=Functional(type="XC", name="LDA", libxc=False),
                                 HARTREE=Functional(type="HARTREE"), PSEUDO=PP)
            rho0 = DirectField(grid=grid1)
            rho0[:] = 12.0 / grid1.volume
            opt = Optimization(EnergyEvaluator=EE, optimization_method=meth,
                               optimization_options={"econv": 1e-11 * 4, "maxiter": maxiter, "maxfun": 50})
            with contextlib.redirect_stdout(io.StringIO()):
                r = opt.optimize_rho(guess_rho=rho0)
            key = "%s_%s_" % (meth.replace("-", ""), tag)
            out[key + "maxiter"] = maxiter
            out[key + "E"] = float(EE.Energy(r))
            out[key + "mu"] = float(opt.mu)
            out[key + "N"] = float(r.integral())
            out[key + "converged"] = int(opt.converged)
            out[key + "niter"] = sum(1 for l in lines if l[:1].isdigit()) - 1
            print(meth, tag, out[key + "E"], out[key + "mu"], out[key + "converged"], out[key + "niter"])
    fn = os.path.join(HERE, "reference_opt.npz")
    np.savez_compressed(fn, **{k: np.asarray(v) for k, v in out.items()})
    print("wrote", fn)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
