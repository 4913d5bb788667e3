"""The oracle's restatement of the two-body WGC kernel (Phys. Rev. B 60, 16350
(1999); no reference implementation, so its parity is unpinned) checked against
its own mathematics: the inverse Lindhard function's first and second
derivatives against central differences, the Taylor coefficients of xi_gamma
against the exact two-body Fermi wave vector, the kernel derivatives against
central differences in k, and the potential against a central difference of
the energy."""
import numpy as np
import pytest

from dftpy_gb300 import synthetic as syn
from oracle import ofdft_np as O


@pytest.mark.parametrize("lo,hi", [(0.05, 0.95), (1.05, 3.6), (3.7, 12.0)])
def test_lindhard_derivatives(lo, hi):
    """eta F' and eta^2 F'' against 50-digit derivatives of the closed form
    (the closed form below 3.65, where the series takes over; the series'
    truncation above it)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50

    def F(e):
        L = mp.mpf("0.5") + mp.mpf("0.25") * (1 - e ** 2) * mp.log((1 + e) / abs(1 - e)) / e
        return 1 / L - 3 * e ** 2 - 1

    eta = np.linspace(lo, hi, 13)
    Fo, d1, d2 = O.lindhard_d2(eta, 1.0, 1.0)
    np.testing.assert_allclose(Fo, O.lindhard(eta, 1.0, 1.0), rtol=1e-13, atol=1e-13)
    ref1 = np.array([float(mp.mpf(e) * mp.diff(F, mp.mpf(e), 1)) for e in eta])
    ref2 = np.array([float(mp.mpf(e) ** 2 * mp.diff(F, mp.mpf(e), 2)) for e in eta])
    np.testing.assert_allclose(d1, ref1, rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(d2, ref2, rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("gamma", [2.7, 1.0, 4.0])
def test_taylor_coefficients_of_xi(gamma):
    c1, c2 = O.wgc_taylor(gamma)
    rng = np.random.default_rng(1)
    for _ in range(20):
        t, tp = rng.uniform(-1, 1, 2) * 1e-2
        exact = (((1 + t) ** (gamma / 3) + (1 + tp) ** (gamma / 3)) / 2) ** (1 / gamma) - 1
        approx = (t + tp) / 6 + c1 * (t * t + tp * tp) + c2 * (t + tp) ** 2
        first = (t + tp) / 6
        # the error is third order in 1e-2, far below the first-order one
        assert abs(exact - approx) <= 1e-7, (exact, approx)
        assert abs(exact - approx) <= 0.05 * abs(exact - first) + 1e-12


def _kernel_at(grid, rho0, k, x, alpha, beta):
    """c (k/k*)^p F(q/2k; x, 1) at any Fermi wave vector k."""
    kstar = (3.0 * rho0 * np.pi ** 2) ** (1.0 / 3.0)
    cTF = 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
    c = 5.0 / (9.0 * alpha * beta * rho0 ** (alpha + beta - 5.0 / 3.0)) * cTF
    p = 5.0 - 3.0 * (alpha + beta)
    return c * (k / kstar) ** p * O.lindhard(grid.q / (2.0 * k), x, 1.0)


@pytest.mark.parametrize("ab", [((5 + 5 ** 0.5) / 6, (5 - 5 ** 0.5) / 6), (0.5, 0.5)])
def test_kernel_derivatives(ab):
    alpha, beta = ab
    lat, _ = syn.fcc_cell(7.6)
    grid = O.Grid(lat, (20, 18, 16))
    rho0, gamma = 0.03, 2.7
    K0, Ka, Kb, Kc = O.wgc_kernels(grid, rho0, 1.0, alpha, beta, gamma)
    kstar = (3.0 * rho0 * np.pi ** 2) ** (1.0 / 3.0)
    h = 1e-4
    Kp = _kernel_at(grid, rho0, kstar * (1 + h), 1.0, alpha, beta)
    K = _kernel_at(grid, rho0, kstar, 1.0, alpha, beta)
    Km = _kernel_at(grid, rho0, kstar * (1 - h), 1.0, alpha, beta)
    K1 = (Kp - Km) / (2 * h)
    K2 = (Kp - 2 * K + Km) / h ** 2
    c1, c2 = O.wgc_taylor(gamma)
    m = np.ones(K.shape, bool)
    m.flat[0] = False
    # points away from the Kohn singularity eta = 1, where the differences do not converge
    eta = grid.q / (2 * kstar)
    m &= np.abs(eta - 1.0) > 0.05
    np.testing.assert_allclose(K0[m], K[m], rtol=1e-13, atol=1e-13)
    # central differences: 1e-8 relative truncation in K1, ~1e-5 rounding in K2
    np.testing.assert_allclose(Ka[m], K1[m] / 6, rtol=1e-6, atol=1e-8)
    np.testing.assert_allclose(Kb[m], (c1 + c2) * K1[m] + K2[m] / 72, rtol=1e-3, atol=1e-5)
    np.testing.assert_allclose(Kc[m], 2 * c2 * K1[m] + 2 * K2[m] / 72, rtol=1e-3, atol=1e-5)


@pytest.mark.parametrize("rho0", [None, 0.025])
def test_potential_is_the_energy_gradient(rho0):
    lat = np.array([[7.4, 0.0, 0.0], [1.1, 7.2, 0.0], [0.5, 0.8, 6.9]])
    nr = (18, 16, 20)
    grid = O.Grid(lat, nr)
    rho = syn.smooth_density(lat, nr, 4.0, seed=3, amp=0.4)
    f = O.WGC(rho0=rho0)
    out = f(rho, grid)
    rng = np.random.default_rng(7)
    d = rng.normal(size=rho.shape) * rho * 0.05
    d -= d.mean()  # the mean density (rho0 of the mean rule) does not move
    h = 1e-5
    Ep = f(rho + h * d, grid, calc=("E",))["E"]
    Em = f(rho - h * d, grid, calc=("E",))["E"]
    fd = (Ep - Em) / (2 * h)
    an = (out["V"] * d).sum() * grid.dV
    assert abs(fd - an) <= 1e-7 * max(1.0, abs(an)), (fd, an)
