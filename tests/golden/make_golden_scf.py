"""Generate tests/golden/reference_scf.npz: the density mixers
(src/dftpy/mixer/pulay.py, linear.py, mixer.py) and the OE-SCF solver
(src/dftpy/optimization/scf.py) computed by the REFERENCE implementation.

Mixers: seeded sequences nin_k -> nout_k = 0.9 nin_k + 0.1 Q_k on a 12x14x16
grid, nine steps per configuration; the final density and per-step checksums.
OE-SCF: fcc Al (4 atoms, 24^3), vW + LDA + Hartree + PME pseudopotential with
the WT nonlocal part (y = 0) frozen as the embedding, Pulay/Kerker mixing;
the energy history and the final density.

Run in a container that has the reference sources:

    python tests/golden/make_golden_scf.py <reference source tree>
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden import make_ions, ref_objects, setup, write_pp  # noqa: E402

MIX_LAT = np.diag([9.0, 8.0, 10.0])
MIX_NR = (12, 14, 16)
MIX_STEPS = 9
# (tag, scheme, kwargs)
MIX_CASES = [
    ("P1", "pulay", dict(predtype=None, maxm=5, coef=0.7, delay=0)),
    ("P2", "pulay", dict(predtype="kerker", predcoef=[1.0, 1.0, 1.0], maxm=7, coef=0.7, delay=2)),
    ("P3", "pulay", dict(predtype="inverse_kerker", predcoef=[0.8], maxm=3, coef=0.5, delay=1, predecut=1.0)),
    ("P4", "pulay", dict(predtype="resta", predcoef=[2.0, 1.0, 3.0], maxm=4, coef=0.6, delay=0, restarted=True,
                         predecut=5.0)),
    ("L1", "linear", dict(predtype="kerker", predcoef=[0.9, 1.2, 0.8], coef=0.4, delay=1)),
    ("L2", "linear", dict(predtype="inverse_kerker", coef=0.7, predecut=1.0)),
]


def mix_inputs():
    """The seeded start density and the targets Q_k (shared with the tests)."""
    from dftpy_gb300 import synthetic as syn
    nin0 = syn.smooth_density(MIX_LAT, MIX_NR, 6.0, seed=30, amp=0.3)
    Q = [syn.smooth_density(MIX_LAT, MIX_NR, 6.0, seed=40 + k, amp=0.5) for k in range(MIX_STEPS)]
    return nin0, Q


def main(ref_root):
    setup(ref_root)
    DirectGrid, DirectField, Ions = ref_objects()
    from dftpy.mixer import Mixer
    from dftpy.mixer.mixer import SpecialPrecondition
    from dftpy.functional import Functional
    from dftpy.functional.total_functional import TotalFunctional
    from dftpy.functional.pseudo import LocalPseudo
    from dftpy.functional.external_potential import ExternalPotential
    from dftpy.optimization import Optimization, OESCF
    from dftpy_gb300 import synthetic as syn

    out = {}
    grid = DirectGrid(lattice=MIX_LAT, nr=MIX_NR, full=False)
    nin0, Q = mix_inputs()
    for tag, scheme, kw in MIX_CASES:
        mixer = Mixer(scheme=scheme, **{k: (list(v) if isinstance(v, list) else v) for k, v in kw.items()})
        nin = DirectField(grid=grid, data=nin0.copy())
        sums = []
        for k in range(MIX_STEPS):
            nout = DirectField(grid=grid, data=0.9 * np.asarray(nin) + 0.1 * Q[k])
            nin = mixer(nin, nout)
            a = np.asarray(nin)
            sums.append([a.sum(), (a * a).sum(), (a * Q[0]).sum()])
        out["mix_" + tag + "_final"] = np.asarray(nin)
        out["mix_" + tag + "_sums"] = np.array(sums)
        print(tag, sums[-1])
    # SpecialPrecondition called directly with drho and a residual
    pred = SpecialPrecondition("kerker", [0.9, 1.1, 0.7], predecut=3.0)
    nin = DirectField(grid=grid, data=nin0.copy())
    nout = DirectField(grid=grid, data=Q[0].copy())
    drho = 0.05 * (Q[1] - Q[2])
    res = 0.3 * (Q[3] - nin0)
    out["pred_direct"] = np.asarray(pred(nin, nout, drho=drho, residual=res, coef=0.45))
    out["pred_resonly"] = np.asarray(pred(nin, nout, residual=res))
    # ExternalPotential
    v = syn.smooth_density(MIX_LAT, MIX_NR, 3.0, seed=50, amp=0.6) - 0.2
    ext = ExternalPotential(v=DirectField(grid=grid, data=v))
    out["ext_E"] = float(ext(DirectField(grid=grid, data=nin0.copy()), calcType={"E"}).energy)

    # ---- OE-SCF ------------------------------------------------------------
    tmp = tempfile.mkdtemp()
    ppA = write_pp(tmp, "Al", 3.0, 1.0)
    lat, pos = syn.fcc_cell(7.6)
    pos = pos + np.random.default_rng(11).normal(0, 0.1, pos.shape)
    ions = make_ions(Ions, lat, pos, ["Al"] * 4, 3.0)
    g2 = DirectGrid(lattice=lat, nr=(24, 24, 24), full=False)
    PP = LocalPseudo(grid=g2, ions=ions, PP_list={"Al": ppA}, PME=True)
    XC = Functional(type="XC", name="LDA", libxc=False)
    HA = Functional(type="HARTREE")
    EE = TotalFunctional(KineticEnergyFunctional=Functional(type="KEDF", name="vW"), XCFunctional=XC, HARTREE=HA,
                         PSEUDO=PP)
    emb = TotalFunctional(KEDF_EMB=Functional(type="KEDF", name="WT", y=0.0))
    rho0 = DirectField(grid=g2)
    rho0[:] = 12.0 / g2.volume
    opt = Optimization(EnergyEvaluator=EE, optimization_method="CG-HS",
                       optimization_options={"econv": 1e-6 * 4, "maxiter": 100})
    mixer = Mixer(scheme="pulay", predtype="kerker", predcoef=[1.0, 1.0, 1.0], maxm=7, coef=0.7, delay=2)
    sc = OESCF(optimization=opt, evaluator_emb=emb, mixer=mixer)
    rho = sc.optimize_rho(guess_rho=rho0)
    out["scf_lattice"], out["scf_pos"] = lat, pos
    out["scf_energy_history"] = np.array([float(e) for e in sc.energyhistory])
    out["scf_iter"] = int(sc.iter)
    out["scf_rho"] = np.asarray(rho)
    out["scf_econv_final"] = float(opt.optimization_options["econv"])
    print("OESCF", out["scf_energy_history"], sc.iter)
    np.savez_compressed(os.path.join(HERE, "reference_scf.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
