"""The two-body WGC kernel on the device (ofdft_wgc_*) against the oracle's
restatement of the published algorithm (Phys. Rev. B 60, 16350 (1999)).  The
reference has no implementation, so parity is unpinned: the oracle itself is
checked against its own mathematics in tests/test_oracle_wgc.py.  Bars (FP64):
energy within 1e-10 relative, potential within 1e-9 a.u. max-abs; FP32 within
2e-6 relative in energy and 1e-5 of max|V| in potential; the potential is the
gradient of the energy (a central difference at 64^3)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D
from dftpy_gb300 import synthetic as syn
from oracle import ofdft_np as O

LAT = np.array([[7.4, 0.0, 0.0], [1.1, 7.2, 0.0], [0.5, 0.8, 6.9]])


@pytest.mark.parametrize("rho0", [None, 0.025])
@pytest.mark.parametrize("gamma", [2.7, 1.5])
def test_wgc_matches_oracle(rho0, gamma):
    torch.cuda.set_device(0)
    nr = (24, 20, 18)
    rho_np = syn.smooth_density(LAT, nr, 4.0, seed=3, amp=0.4)
    grid = D.DirectGrid(LAT, nr)
    rho = D.DirectField(grid, data=rho_np)
    f = D.Functional(type="KEDF", name="WGC-NL", gamma=gamma, rho0=rho0)
    out = f(rho)
    ref = O.WGC(gamma=gamma, rho0=rho0)(rho_np, O.Grid(LAT, nr))
    assert abs(out.energy - ref["E"]) <= 1e-10 * max(1.0, abs(ref["E"])), (out.energy, ref["E"])
    assert float(np.abs(out.potential.numpy() - ref["V"]).max()) <= 1e-9
    # the same bits on a second call; FP32 within the mixed-precision bars
    assert f(rho).energy == out.energy
    r32 = D.DirectField(grid, data=rho_np, dtype=torch.float32)
    o32 = f(r32)
    assert abs(o32.energy - ref["E"]) <= 2e-6 * max(1.0, abs(ref["E"]))
    v32 = o32.potential.as_subclass(torch.Tensor).double().cpu().numpy()
    assert float(np.abs(v32 - ref["V"]).max()) <= 1e-5 * float(np.abs(ref["V"]).max())


def test_wgc_kedf_is_tfvw_plus_nonlocal():
    torch.cuda.set_device(0)
    nr = (24, 20, 18)
    grid = D.DirectGrid(LAT, nr)
    rho = D.DirectField(grid, data=syn.smooth_density(LAT, nr, 4.0, seed=4, amp=0.3))
    full = D.Functional(type="KEDF", name="WGC")(rho)
    parts = D.Functional(type="KEDF", name="TFVW")(rho) + D.Functional(type="KEDF", name="WGC-NL")(rho)
    assert abs(full.energy - parts.energy) <= 1e-12 * abs(parts.energy)
    assert torch.equal(full.potential.as_subclass(torch.Tensor), parts.potential.as_subclass(torch.Tensor))
    split = D.Functional(type="KEDF", name="WGC").compute(rho, split=True)
    assert set(split) >= {"TF", "VW", "WGC-NL"}


def test_wgc_potential_is_energy_gradient_64():
    torch.cuda.set_device(0)
    lat, pos = syn.fcc_supercell(7.6, 2, sigma=0.1, seed=3)
    nr = (64, 64, 64)
    rho_np = syn.atomic_density(lat, nr, pos, [3.0] * len(pos), width=1.4, floor=0.002)
    grid = D.DirectGrid(lat, nr)
    f = D.Functional(type="KEDF", name="WGC-NL")
    rho = D.DirectField(grid, data=rho_np)
    out = f(rho)
    d = np.random.default_rng(5).normal(size=rho_np.shape) * rho_np * 0.05
    d -= d.mean()
    h = 1e-5
    Ep = f(D.DirectField(grid, data=rho_np + h * d), calcType={"E"}).energy
    Em = f(D.DirectField(grid, data=rho_np - h * d), calcType={"E"}).energy
    fd = (Ep - Em) / (2 * h)
    an = float((out.potential.numpy() * d).sum() * grid.dV)
    assert abs(fd - an) <= 1e-7 * max(1.0, abs(an)), (fd, an)
