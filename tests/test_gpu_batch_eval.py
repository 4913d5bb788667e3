"""The persistent batched evaluation (one cooperative launch for every system
of a batch) against each system's own evaluation through TotalFunctional.

Systems: seven cells of the batching workload (fcc/bcc/sc Al, grids from
{48, 64, 72, 80, 96}^3) plus a non-orthogonal cell on a 40 x 36 x 30 grid
(radices 8, 5; 4, 3, 3; 2, 3, 5, and a non-orthogonal G^2), TF + vW + LDA +
Hartree + PME local PP, seeded smooth densities.  Bars: FP64 energy within
1e-10 relative (per-atom scale), potential within 1e-9 a.u. max-abs.  FP32
against the FP64 single-system result: energy within 2e-6 relative, and the
potential error no larger than twice that of the FP32 single-system path
(cuFFT) or 1e-5 of max|V|, whichever is larger (the vW term multiplies the
float32 transform round-off by G^2, so both FP32 paths sit near 1e-4 of
max|V| pointwise).  Repeated runs give the same bits; inactive systems
are left untouched; every autotuned or stored shape gives the same energies to
rounding."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn
from dftpy_gb300.batch import BatchEvaluator


def _systems(dtype):
    gp, vp = syn.analytic_vloc(3.0, 1.0)
    specs = syn.batch_systems(7, seed=5)
    lat = np.array([[7.4, 0.0, 0.0], [1.3, 7.1, 0.0], [0.6, 0.9, 6.8]])
    pos = np.random.default_rng(3).uniform(0, 1, (4, 3)) @ lat
    specs.append({"lattice": lat, "positions": pos, "nr": (40, 36, 30), "kind": "triclinic"})
    out = []
    for k, sd in enumerate(specs):
        lat, pos, nr = sd["lattice"], sd["positions"], tuple(sd["nr"])
        nat = len(pos)
        grid = D.DirectGrid(lat, nr)
        ions = D.Ions(symbols=["Al"] * nat, positions=pos, cell=lat)
        pp = D.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": D.functional.RECPOT(r=gp, v=vp, zval=3)}, PME=True)
        tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="TFVW"),
                                XCFunctional=D.Functional(type="XC", name="LDA"),
                                HARTREE=D.Functional(type="HARTREE"), PSEUDO=pp)
        rho = D.DirectField(grid, data=syn.smooth_density(lat, nr, 3.0 * nat, seed=10 + k, amp=0.4), dtype=dtype)
        out.append((nat, grid, tot, rho))
    return out


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batch_matches_single_system_evaluations(dtype):
    torch.cuda.set_device(0)
    sy = _systems(dtype)
    be = BatchEvaluator([t for _, _, t, _ in sy], [g for _, g, _, _ in sy], dtype=dtype, tune=True)
    outs = be([r for _, _, _, r in sy])
    shape = be.shape
    assert shape["block"] in (128, 256) and shape["tuned_ms"] > 0
    for (nat, grid, tot, rho), o in zip(sy, outs):
        v = o.potential.as_subclass(torch.Tensor).double()
        if dtype == torch.float64:
            ref = tot(rho)
            vr = ref.potential.as_subclass(torch.Tensor)
            assert abs(o.energy - ref.energy) <= 1e-10 * max(nat, abs(ref.energy)), (o.energy, ref.energy)
            assert float((v - vr).abs().max()) <= 1e-9
        else:
            ref = tot(D.DirectField(grid, data=rho.as_subclass(torch.Tensor).double()))
            vr = ref.potential.as_subclass(torch.Tensor)
            single = tot(rho).potential.as_subclass(torch.Tensor).double()
            e_single = float((single - vr).abs().max())
            assert abs(o.energy - ref.energy) <= 2e-6 * abs(ref.energy), (o.energy, ref.energy)
            assert float((v - vr).abs().max()) <= max(2.0 * e_single, 1e-5 * float(vr.abs().max())), \
                (float((v - vr).abs().max()), e_single)
    # the same bits on a second run
    again = be([r for _, _, _, r in sy])
    for a, b in zip(outs, again):
        assert a.energy == b.energy


def test_batch_inactive_systems_untouched_and_shapes_agree():
    torch.cuda.set_device(0)
    sy = _systems(torch.float64)
    be = BatchEvaluator([t for _, _, t, _ in sy], [g for _, g, _, _ in sy], tune=False)
    rhos = [r for _, _, _, r in sy]
    base = be(rhos)
    vs = [torch.full_like(r.as_subclass(torch.Tensor), 7.0) for r in rhos]
    active = [k % 2 == 0 for k in range(len(rhos))]
    part = be(rhos, active=active, out=vs)
    for k, (a, b) in enumerate(zip(base, part)):
        if active[k]:
            assert a.energy == b.energy
        else:
            assert b is None and bool((vs[k] == 7.0).all())
    import ctypes as C
    from dftpy_gb300 import _lib
    for block, rows, lines in ((128, 2, 8), (256, 8, 32)):
        _lib.check(_lib.load().ofdft_batch_eval_set_shape(be._h, block, rows, lines))
        for (nat, _, _, _), a, b in zip(sy, base, be(rhos)):
            assert abs(a.energy - b.energy) <= 1e-12 * max(nat, abs(a.energy))


def test_batch_tuning_table_round_trip(tmp_path):
    torch.cuda.set_device(0)
    sy = _systems(torch.float32)[:3]
    fn = str(tmp_path / "tune.json")
    be = BatchEvaluator([t for _, _, t, _ in sy], [g for _, g, _, _ in sy], dtype=torch.float32, tuning_table=fn)
    be([r for _, _, _, r in sy])
    import json
    table = json.load(open(fn))
    assert be.signature in table
    be2 = BatchEvaluator([t for _, _, t, _ in sy], [g for _, g, _, _ in sy], dtype=torch.float32, tuning_table=fn)
    be2([r for _, _, _, r in sy])
    assert {k: be2.shape[k] for k in ("block", "rows", "lines")} == {k: table[be.signature][k]
                                                                    for k in ("block", "rows", "lines")}


def test_batch_refuses_ineligible_systems():
    """An axis with a factor other than 2, 3 and 5, or a functional beyond TF, vW,
    LDA, Hartree and the local PP, is refused at construction with a clear error."""
    torch.cuda.set_device(0)
    lat = np.diag([7.6, 7.6, 7.6])
    g28 = D.DirectGrid(lat, (28, 32, 32))
    tot = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="TFVW"),
                            XCFunctional=D.Functional(type="XC", name="LDA"), HARTREE=D.Functional(type="HARTREE"))
    with pytest.raises(NotImplementedError):
        BatchEvaluator([tot], [g28])
    g32 = D.DirectGrid(lat, (32, 32, 32))
    wt = D.TotalFunctional(KineticEnergyFunctional=D.Functional(type="KEDF", name="WT"),
                           HARTREE=D.Functional(type="HARTREE"))
    with pytest.raises(NotImplementedError):
        BatchEvaluator([wt], [g32])
