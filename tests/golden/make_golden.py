"""Generate the golden fixtures under tests/golden/ by running the REFERENCE
implementation (Quantum-MultiScale/DFTpy) on seeded inputs.

Run in a container that has the reference sources:

    python tests/golden/make_golden.py <reference source tree>

The reference needs ASE, which is not installed here; oracle/ase_shim provides
the few members it uses.  Nothing else in the repository reads the reference
at run time: tests compare against the .npz files this script writes.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def setup(ref_root):
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    sys.dont_write_bytecode = True
    sys.path.insert(0, os.path.join(REPO, "oracle", "ase_shim"))
    sys.path.insert(0, os.path.join(ref_root, "src"))
    sys.path.insert(0, REPO)


def ref_objects():
    from dftpy.grid import DirectGrid
    from dftpy.field import DirectField
    from dftpy.ions import Ions
    return DirectGrid, DirectField, Ions


def make_ions(Ions, lattice, pos, symbols, zval):
    ions = Ions(symbols=symbols, positions=pos, cell=lattice)
    ions.set_charges(zval)
    return ions


def write_pp(tmp, name, Z, rc):
    from dftpy_gb300.synthetic import analytic_vloc
    from oracle.ofdft_np import write_recpot
    g, v = analytic_vloc(Z, rc)
    fn = os.path.join(tmp, name + ".recpot")
    write_recpot(fn, g[-1], v, header="analytic Z=%g rc=%g" % (Z, rc))
    return fn


def terms_on(DirectGrid, DirectField, lattice, nr, rho_arr, ions, pp_list, prefix, out, lwt_cfgs=(), full_v=True):
    from dftpy.functional import Functional
    from dftpy.functional.pseudo import LocalPseudo
    from dftpy.functional.kedf import KEDF
    grid = DirectGrid(lattice=lattice, nr=nr, full=False)
    rho = DirectField(grid=grid, data=rho_arr.copy())
    res = {}
    res["TF"] = Functional(type="KEDF", name="TF")(rho.copy())
    res["VW"] = Functional(type="KEDF", name="VW")(rho.copy())
    res["WTNL"] = KEDF(name="WT-NL")(rho.copy())
    res["XC"] = Functional(type="XC", name="LDA", libxc=False)(rho.copy())
    res["H"] = Functional(type="HARTREE")(rho.copy())
    if ions is not None:
        pme = LocalPseudo(grid=grid, ions=ions, PP_list=pp_list, PME=True)
        res["PPPME"] = pme(rho.copy())
        out[prefix + "F_PPPME"] = np.asarray(pme.forces(rho.copy()))
        exact = LocalPseudo(grid=grid, ions=ions, PP_list=pp_list, PME=False)
        res["PPEX"] = exact(rho.copy())
        out[prefix + "F_PPEX"] = np.asarray(exact.forces(rho.copy()))
    for tag, kw in lwt_cfgs:
        res[tag] = KEDF(name="LWT-NL", **kw)(rho.copy())
    for k, o in res.items():
        out[prefix + "E_" + k] = float(o.energy)
        if full_v:
            out[prefix + "V_" + k] = np.asarray(o.potential)
    return grid, rho


def edge_density(lattice, nr, positions, zvals, width):
    """The B block's density, pinned here (not taken from dftpy_gb300.synthetic,
    whose generator may change): periodic Gaussians summed over the whole grid
    by minimum image, normalised to sum(zvals) electrons.  Reproduces the
    stored B_rho bit for bit."""
    s = [np.arange(n) / n for n in nr]
    S = np.stack(np.meshgrid(*s, indexing="ij"), axis=-1)
    inv = np.linalg.inv(lattice)
    rho = np.zeros(tuple(nr), dtype=np.float64)
    for p, z in zip(positions, zvals):
        f = S - (p @ inv)
        f -= np.round(f)
        r = f @ lattice
        rr = (r * r).sum(-1)
        rho += z * np.exp(-rr / (2 * width ** 2)) / (2 * np.pi * width ** 2) ** 1.5
    vol = abs(np.linalg.det(lattice))
    rho *= float(np.sum(zvals)) / (rho.sum() * vol / rho.size)
    return rho


def main(ref_root):
    setup(ref_root)
    DirectGrid, DirectField, Ions = ref_objects()
    from dftpy.ewald import ewald
    from dftpy.functional.pseudo.recpot import RECPOT
    from dftpy.functional import Functional
    from dftpy.functional.total_functional import TotalFunctional
    from dftpy.functional.pseudo import LocalPseudo
    from dftpy.optimization import Optimization
    from dftpy.formats import io as dio
    from dftpy_gb300 import synthetic as syn

    tmp = tempfile.mkdtemp()
    ppA = write_pp(tmp, "Al", 3.0, 1.0)
    ppB = write_pp(tmp, "Mg", 2.0, 1.2)
    out = {}

    # ---- recpot reader on our synthetic file --------------------------------
    rp = RECPOT(ppA)
    out["recpot_gp"] = np.asarray(rp.r)
    out["recpot_vp"] = np.asarray(rp.v)
    out["recpot_zval"] = float(rp.zval)
    with open(ppA) as f:
        out["recpot_text"] = np.frombuffer(f.read().encode(), dtype=np.uint8)

    wgc = dict(alpha=(5 + np.sqrt(5)) / 6, beta=(5 - np.sqrt(5)) / 6)
    # ---- A: fields on a small anisotropic grid, fcc Al 4 atoms -------------
    lat, pos = syn.fcc_cell(7.6)
    pos = pos + np.random.default_rng(11).normal(0, 0.1, pos.shape)
    nr = (24, 20, 18)
    rhoA = syn.smooth_density(lat, nr, 12.0, seed=3, amp=0.4)
    ions = make_ions(Ions, lat, pos, ["Al"] * 4, 3.0)
    out["A_lattice"], out["A_pos"], out["A_nr"], out["A_rho"] = lat, pos, np.array(nr), rhoA
    lwt = [("LWT64", dict(nsp=64, kdd=3, interp="linear", **wgc)),
           ("LWT8H", dict(nsp=8, kdd=3, interp="hermite", **wgc)),
           ("LWTR", dict(ratio=1.15, kdd=3, interp="linear")),
           ("LWT8K1", dict(nsp=8, kdd=1, interp="linear", **wgc))]
    terms_on(DirectGrid, DirectField, lat, nr, rhoA, ions, {"Al": ppA}, "A_", out, lwt)
    ew = ewald(ions=ions, grid=DirectGrid(lattice=lat, nr=nr, full=False), PME=True)
    out["A_ewald_eta"] = ew.eta
    out["A_ewald_E"] = ew.energy
    out["A_ewald_F"] = np.asarray(ew.forces)
    out["A_ewald_Ecorr"] = ew.Energy_corr()
    out["A_ewald_Erec"] = ew.Energy_rec_PME()
    out["A_ewald_Ereal"] = ew.Energy_real_fast2()
    ewd = ewald(ions=ions, grid=DirectGrid(lattice=lat, nr=nr, full=False), PME=False)
    out["A_ewaldex_E"] = ewd.energy
    out["A_ewaldex_F"] = np.asarray(ewd.forces)

    # ---- B: edge densities (tiny, zero and negative values) ----------------
    latB = np.diag([9.0, 8.0, 10.0])
    posB = np.array([[1.0, 1.0, 1.0], [5.5, 4.0, 6.0]])
    nrB = (16, 18, 20)
    rhoB = edge_density(latB, nrB, posB, [3.0, 3.0], width=0.9)
    rhoB[0, 0, 0] = -1e-5
    rhoB[1, 2, 3] = 0.0
    out["B_lattice"], out["B_nr"], out["B_rho"] = latB, np.array(nrB), rhoB
    lwtB = [("LWT16", dict(nsp=16, kdd=3, interp="linear", **wgc)),
            ("LWT6H", dict(nsp=6, kdd=3, interp="hermite"))]
    terms_on(DirectGrid, DirectField, latB, nrB, rhoB, None, None, "B_", out, lwtB)

    # ---- C: c1 workload (fcc Al, 32^3, TFVW+LDA+H+PP) -- energies and ground state
    lat1, pos1 = syn.fcc_cell(7.60)
    ions1 = make_ions(Ions, lat1, pos1, ["Al"] * 4, 3.0)
    grid1 = DirectGrid(lattice=lat1, nr=(32, 32, 32), full=False)
    ew1 = ewald(ions=ions1, grid=grid1, PME=True)
    out["C_ewald_E"] = ew1.energy
    out["C_ewald_F"] = np.asarray(ew1.forces)
    for meth in ("TN", "LBFGS", "CG-HS"):
        grid1 = DirectGrid(lattice=lat1, nr=(32, 32, 32), full=False)
        ions1 = make_ions(Ions, lat1, pos1, ["Al"] * 4, 3.0)
        PP = LocalPseudo(grid=grid1, ions=ions1, PP_list={"Al": ppA}, PME=True)
        KE = Functional(type="KEDF", name="TFVW")
        XC = Functional(type="XC", name="LDA", libxc=False)
        HA = Functional(type="HARTREE")
        EE = TotalFunctional(KineticEnergyFunctional=KE, XCFunctional=XC, HARTREE=HA, PSEUDO=PP)
        rho0 = DirectField(grid=grid1)
        rho0[:] = 12.0 / grid1.volume
        opt = Optimization(EnergyEvaluator=EE, optimization_method=meth,
                           optimization_options={"econv": 1e-11 * 4, "maxiter": 60, "maxfun": 50})
        r = opt.optimize_rho(guess_rho=rho0)
        tag = "C_" + meth.replace("-", "") + "_"
        out[tag + "E"] = float(EE.Energy(r))
        out[tag + "mu"] = float(opt.mu)
        out[tag + "converged"] = int(opt.converged)
        res = (opt.functional.potential - opt.mu) * opt.phi
        out[tag + "dP"] = float((res * res).sum() * grid1.dV)
        if meth == "TN":
            out[tag + "rho"] = np.asarray(r)
            out["C_F_PP"] = np.asarray(PP.forces(r))

    # ---- D: 32-atom WT system with PME forces (Ewald + PP), 2 species ------
    latD, posD = syn.fcc_supercell(7.6, (2, 2, 2), sigma=0.1, seed=5)
    symD = ["Al" if i % 2 == 0 else "Mg" for i in range(len(posD))]
    ionsD = make_ions(Ions, latD, posD, symD, {"Al": 3.0, "Mg": 2.0})
    nrD = (40, 40, 40)
    gridD = DirectGrid(lattice=latD, nr=nrD, full=False)
    nel = 3.0 * symD.count("Al") + 2.0 * symD.count("Mg")
    rhoD = syn.smooth_density(latD, nrD, nel, seed=9, amp=0.25)
    PPD = LocalPseudo(grid=gridD, ions=ionsD, PP_list={"Al": ppA, "Mg": ppB}, PME=True)
    rd = DirectField(grid=gridD, data=rhoD.copy())
    out["D_lattice"], out["D_pos"], out["D_nr"], out["D_rho"] = latD, posD, np.array(nrD), rhoD
    out["D_species"] = np.array([0 if s == "Al" else 1 for s in symD])
    out["D_E_PP"] = float(PPD(rd).energy)
    out["D_F_PP"] = np.asarray(PPD.forces(rd))
    ewD = ewald(ions=ionsD, grid=gridD, PME=True)
    out["D_ewald_E"] = ewD.energy
    out["D_ewald_F"] = np.asarray(ewD.forces)
    KED = Functional(type="KEDF", name="WT")
    out["D_E_WT"] = float(KED(rd.copy()).energy)

    # ---- E: the reference's own fixture (Al_fde_rho.pp) and goldens --------
    data = os.path.join(ref_root, "examples", "DATA")
    ionsE, rhoF, _ = dio.read_all(os.path.join(data, "Al_fde_rho.pp"))
    # the reader builds a full complex grid; the reference's default path (and ours)
    # is the half grid (gfull=False), so evaluate on a half grid with the same data.
    out["E_E_WT_fullgrid"] = float(Functional(type="KEDF", name="WT")(rhoF.copy()).energy)
    gridE = DirectGrid(lattice=rhoF.grid.lattice, nr=rhoF.grid.nrR, full=False)
    rhoE = DirectField(grid=gridE, data=np.asarray(rhoF).copy())
    out["E_lattice"] = np.asarray(rhoE.grid.lattice)
    out["E_nr"] = np.asarray(rhoE.grid.nrR)
    out["E_rho"] = np.asarray(rhoE)
    out["E_pos"] = np.asarray(ionsE.positions)
    out["E_E_WT"] = float(Functional(type="KEDF", name="WT")(rhoE.copy()).energy)
    for nm in ("al.lda.recpot", "Al_lda.oe01.recpot"):
        r = RECPOT(os.path.join(data, nm))
        key = "E_pp_" + nm.split(".")[0].replace("_", "")
        out[key + "_gp"] = np.asarray(r.r)
        out[key + "_vp"] = np.asarray(r.v)
        out[key + "_zval"] = float(r.zval)
    PPE = LocalPseudo(grid=rhoE.grid, ions=ionsE, PP_list={"Al": os.path.join(data, "al.lda.recpot")})
    out["E_E_PP_allda"] = float(PPE(rhoE).energy)
    ewE = ewald(rho=rhoE, ions=ionsE, PME=True)
    out["E_ewald_E"] = ewE.energy
    out["E_ewald_Ecorr"] = ewE.Energy_corr()
    out["E_ewald_Erec"] = ewE.Energy_rec_PME()
    out["E_ewald_F"] = np.asarray(ewE.forces)

    fn = os.path.join(HERE, "reference_golden.npz")
    np.savez_compressed(fn, **{k: np.asarray(v) for k, v in out.items()})
    print("wrote", fn, os.path.getsize(fn), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the reference source tree>" % sys.argv[0])
    main(sys.argv[1])
