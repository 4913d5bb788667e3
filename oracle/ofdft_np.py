"""numpy restatement of the reference OF-DFT hot path (TEST INFRASTRUCTURE ONLY).

This module is the oracle the CUDA path is checked against.  It is our own
restatement of the algorithms in Quantum-MultiScale/DFTpy; every function
names the reference file:line it follows.  The reference computes in float64
/ complex128 throughout, and so does this module.  Third-party calls the
reference makes (numpy pocketfft, scipy FITPACK splrep/splev, scipy.special
erfc/erfcinv, scipy's MINPACK-2 line search) are made here too, so that the
oracle's arithmetic is the reference's arithmetic.

Conventions (reference src/dftpy/field.py:413-430, :779-804):
  * a real field is a C-ordered (n0, n1, n2) float64 array;
  * ``fft(f)`` = numpy ``rfftn(f) * dV``; ``ifft(F)`` = ``irfftn(F, s=nr) / dV``;
  * G vectors: integer fftfreq indices times the reciprocal lattice
    ``2*pi*inv(lattice).T`` (src/dftpy/grid.py:384-415, :584-620).
"""
import math

import numpy as np
from scipy import special as sp
from scipy.interpolate import splev, splrep

C_TF = 2.87123400018819181594      # src/dftpy/constants.py:82
ZERO = 1e-30                        # src/dftpy/constants.py:85

# CODATA-2014 Bohr (Angstrom) and Hartree (eV), as ase.units derives them.
_e, _me, _hp = 1.6021766208e-19, 9.10938356e-31, 6.626070040e-34
_eps0 = 1.0 / (4.0e-7 * math.pi) / 299792458.0 ** 2
_hbar = _hp / (2.0 * math.pi)
BOHR = 4.0e10 * math.pi * _eps0 * _hbar ** 2 / _me / _e ** 2
HARTREE = _me * _e ** 3 / 16.0 / math.pi ** 2 / _eps0 ** 2 / _hbar ** 2


# --------------------------------------------------------------------------
# grid
# --------------------------------------------------------------------------
class Grid:
    """Direct grid + half-complex reciprocal grid (src/dftpy/grid.py:8-60, :480-620)."""

    def __init__(self, lattice, nr):
        self.lattice = np.asarray(lattice, dtype=np.float64).reshape(3, 3)
        self.nr = np.array(nr, dtype=np.int64)
        self.nnr = int(np.prod(self.nr))
        self.volume = abs(float(np.linalg.det(self.lattice)))
        self.dV = self.volume / self.nnr
        self.nrG = self.nr.copy()
        self.nrG[-1] = self.nr[-1] // 2 + 1
        # reciprocal lattice, rows b_j (grid.py:384-415)
        self.rlattice = (2.0 * np.pi * np.linalg.inv(self.lattice)).T
        self._g = None
        self._gg = None
        self._mask = None

    @property
    def g(self):
        if self._g is None:  # grid.py:584-620 (fftfreq on axes 0,1; rfftfreq on axis 2)
            ax = [np.fft.fftfreq(self.nr[0], d=1.0 / self.nr[0]),
                  np.fft.fftfreq(self.nr[1], d=1.0 / self.nr[1]),
                  np.fft.rfftfreq(self.nr[2], d=1.0 / self.nr[2])]
            S = np.asarray(np.meshgrid(*ax, indexing="ij"))
            self._g = np.einsum("j...,jk->k...", S, self.rlattice)
        return self._g

    @property
    def gg(self):
        if self._gg is None:  # grid.py:523-530
            g = self.g
            self._gg = np.einsum("lijk,lijk->ijk", g, g)
        return self._gg

    @property
    def q(self):
        return np.sqrt(self.gg)  # grid.py:517-521

    @property
    def invgg(self):
        gg = self.gg.copy()  # grid.py:532-541: G=0 -> 0
        gg[0, 0, 0] = 1.0
        inv = 1.0 / gg
        inv[0, 0, 0] = 0.0
        return inv

    @property
    def mask(self):
        """Half-space mask that counts each +-G pair once (grid.py:658-695, serial case)."""
        if self._mask is None:
            nr = self.nr
            D = nr // 2
            M = nr % 2
            m = np.ones(tuple(self.nrG), dtype=bool)
            m[0, D[1] + 1:, 0] = False
            m[D[0] + 1:, :, 0] = False
            if M[2] == 0:
                m[0, 0, D[2]] = False
                m[0, D[1] + 1:, D[2]] = False
                m[D[0] + 1:, :, D[2]] = False
                if M[1] == 0:
                    m[0, D[1], D[2]] = False
                if M[0] == 0:
                    m[D[0], 0, D[2]] = False
                    m[D[0], D[1] + 1:, D[2]] = False
            if M[0] == 0:
                m[D[0], D[1] + 1:, 0] = False
                if M[1] == 0:
                    m[D[0], D[1], 0] = False
            if M[1] == 0:
                m[0, D[1], 0] = False
            if np.all(M == 0):
                m[D[0], D[1], D[2]] = False
            self._mask = m
        return self._mask

    def guess_ecut(self):
        """grid.py:363-366 with RPgrid.g2max = 2*ecut (grid.py:722-723)."""
        lengths = np.sqrt((self.lattice ** 2).sum(axis=1))
        sp1 = lengths / self.nr
        sp2 = lengths / (self.nr - 1)
        spacing = 0.5 * (sp1 + sp2)
        return np.pi ** 2 / (2 * spacing.max() ** 2)


_FFT_WORKERS = None


def set_fft_workers(n):
    """Run the oracle's FFTs on n threads (scipy.fft) instead of numpy's single
    thread; the transforms are the same pocketfft algorithm."""
    global _FFT_WORKERS
    _FFT_WORKERS = n


def fft(f, grid):
    """DirectField.fft: rfftn times dV (field.py:413-430)."""
    if _FFT_WORKERS:
        import scipy.fft as sfft
        return sfft.rfftn(f, workers=_FFT_WORKERS) * grid.dV
    return np.fft.rfftn(f) * grid.dV


def ifft(F, grid):
    """ReciprocalField.ifft(force_real=True): irfftn / dV (field.py:779-804)."""
    if _FFT_WORKERS:
        import scipy.fft as sfft
        return sfft.irfftn(F, s=tuple(grid.nr), axes=(0, 1, 2), workers=_FFT_WORKERS) / grid.dV
    return np.fft.irfftn(F, s=tuple(grid.nr), axes=(0, 1, 2)) / grid.dV


# --------------------------------------------------------------------------
# KEDF: TF, vW
# --------------------------------------------------------------------------
def tf(rho, grid, x=1.0, calc=("E", "V")):
    """Thomas-Fermi (kedf/tf.py:13-35, :66-80); PowerInt(rho,5,3) = cbrt(rho^5) (math_utils.py:158)."""
    out = {}
    if "E" in calc:
        r5 = rho * rho * rho * rho * rho
        ed = np.cbrt(r5) * ((3.0 / 10.0) * (3.0 * np.pi ** 2) ** (2.0 / 3.0))
        out["E"] = ed.sum() * grid.dV * x
    if "V" in calc:
        fac = (3.0 / 10.0) * (5.0 / 3.0) * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
        out["V"] = fac * np.cbrt(rho * rho) * x
    return out


def vw(rho, grid, y=1.0, calc=("E", "V"), sigma=None):
    """von Weizsaecker (kedf/vw.py:29-53 potential, :84-94 energy, :115-131);
    sigma: the Laplacian times exp(-G^2 sigma^2/4) (:45-48)."""
    tol = 1e-30
    rhom = rho.copy()
    rhom[~(rho > 0)] = tol
    sq = np.sqrt(rhom)
    if sigma is None:
        a = ifft(fft(sq, grid) * grid.gg, grid) * 0.5
    else:
        a = ifft(fft(sq, grid) * np.exp(-grid.gg * sigma ** 2 / 4.0) * grid.gg, grid) * 0.5
    sq[np.abs(sq) < tol] = tol
    pot = a / sq
    out = {}
    if "E" in calc:
        m = rho > 0
        out["E"] = np.einsum("i,i->", rho[m], pot[m]) * grid.dV * y
    if "V" in calc:
        out["V"] = pot * y
    return out


# --------------------------------------------------------------------------
# XC: LDA (Slater + Perdew-Zunger 81)
# --------------------------------------------------------------------------
PZ = dict(a=0.0311, b=-0.048, c=0.0020, d=-0.0116, gamma=-0.1423, beta1=1.0529, beta2=0.3334)


def lda(rho, grid, calc=("E", "V")):
    """Built-in LDA (xc/semilocal_xc.py:283-341), unpolarised branch only."""
    a, b, c, d = PZ["a"], PZ["b"], PZ["c"], PZ["d"]
    gamma, beta1, beta2 = PZ["gamma"], PZ["beta1"], PZ["beta2"]
    rc = np.cbrt(rho)
    rc[rc < 1e-30] = 1e-30
    Rs = np.cbrt(3.0 / (4.0 * np.pi)) / rc
    rs1 = Rs < 1
    rs2 = ~rs1
    Rs2sqrt = np.sqrt(Rs[rs2])
    out = {}
    if "E" in calc:
        ex = -3.0 / 4.0 * np.cbrt(3.0 / np.pi) * rc
        ex[rs1] += a * np.log(Rs[rs1]) + b + c * Rs[rs1] * np.log(Rs[rs1]) + d * Rs[rs1]
        ex[rs2] += gamma / (1.0 + beta1 * Rs2sqrt + beta2 * Rs[rs2])
        out["E"] = np.einsum("ijk,ijk->", ex, rho) * grid.dV
    if "V" in calc:
        pot = np.cbrt(-3.0 / np.pi) * rc
        pot[rs1] += (np.log(Rs[rs1]) * (a + 2.0 / 3 * c * Rs[rs1]) + b - 1.0 / 3 * a
                     + 1.0 / 3 * (2 * d - c) * Rs[rs1])
        pot[rs2] += ((gamma + (7.0 / 6.0 * gamma * beta1) * Rs2sqrt + (4.0 / 3.0 * gamma * beta2 * Rs[rs2]))
                     / (1.0 + beta1 * Rs2sqrt + beta2 * Rs[rs2]) ** 2)
        out["V"] = pot
    return out


# --------------------------------------------------------------------------
# Hartree
# --------------------------------------------------------------------------
def hartree(rho, grid, calc=("E", "V")):
    """Hartree (functional/hartree.py:24-45): v_H(G) = 4 pi rho(G)/G^2, G=0 -> 0."""
    vh = ifft(fft(rho, grid) * grid.invgg * 4 * np.pi, grid)
    out = {"V": vh}
    if "E" in calc:
        out["E"] = np.einsum("ijk,ijk->", vh, rho) * grid.dV / 2.0
    return out


_hartree_fn = hartree


# --------------------------------------------------------------------------
# Lindhard / Wang-Teter
# --------------------------------------------------------------------------
_LARGE = [-0.13714285714285712, -6.39999999999999875e-2, -3.77825602968460128e-2,
          -2.51824061652633074e-2, -1.80879839616166146e-2, -1.36715733124818332e-2,
          -1.07236045520990083e-2, -8.65192783339199453e-3, -7.1372762502456763e-3,
          -5.9945117538835746e-3, -5.10997527675418131e-3, -4.41060829979912465e-3,
          -3.84763737842981233e-3, -3.38745061493813488e-3, -3.00624946457977689e-3]


def lindhard(eta, lbda, mu, tol=1e-10):
    """Inverse Lindhard function, 4 branches (kedf/kernel.py:14-136).

    Branch order matters where conditions overlap: normal, then zero, one,
    large overwrite in that order (kernel.py:26-35)."""
    eta = np.asarray(eta, dtype=np.float64)
    tol2 = tol / 10
    cond0 = (eta > tol2) & (np.abs(eta - 1.0) > tol2)
    cond1 = eta < tol
    cond2 = np.abs(eta - 1.0) < tol
    cond3 = eta > 3.65
    out = eta.copy()
    e = eta[cond0]
    out[cond0] = (1.0 / (0.5 + 0.25 * (1.0 - e ** 2) * np.log((1.0 + e) / np.abs(1.0 - e)) / e)
                  - 3.0 * mu * e ** 2 - lbda)
    e = eta[cond1]
    out[cond1] = 1.0 - lbda + e ** 2 * (1.0 / 3.0 - 3.0 * mu)
    e = eta[cond2]
    out[cond2] = 2.0 - lbda - 3.0 * mu + 20.0 * (e - 1.0)
    e = eta[cond3]
    inv2 = 1.0 / e ** 2
    acc = _LARGE[-1] * inv2
    for coef in _LARGE[-2::-1]:
        acc = inv2 * (coef + acc)
    out[cond3] = 3.0 * (1.0 - mu) * e ** 2 - lbda - 0.6 + acc
    return out


def wt_kernel(grid, rho0, x=1.0, alpha=5.0 / 6.0, beta=5.0 / 6.0):
    """WTKernel (kernel.py:325-334): F(q/2kF0; x, 1) * 5/(9 a b rho0^(a+b-5/3)) * C_TF."""
    tkf = 2.0 * (3.0 * rho0 * np.pi ** 2) ** (1.0 / 3.0)
    cTF = 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
    factor = 5.0 / (9.0 * alpha * beta * rho0 ** (alpha + beta - 5.0 / 3.0)) * cTF
    return lindhard(grid.q / tkf, x, 1.0) * factor


class WT:
    """Wang-Teter nonlocal term (kedf/wt.py:109-132) with the kernel cache of
    wt.py:58-73 (rebuilt when rho0 moves by more than 1e-6 or the shape changes)."""

    def __init__(self, x=1.0, alpha=5.0 / 6.0, beta=5.0 / 6.0, rho0=None):
        self.x, self.alpha, self.beta, self.rho0 = x, alpha, beta, rho0
        self._saved_rho0 = 0.0
        self._shape = None
        self._kernel = None

    def kernel(self, rho, grid):
        rho0 = self.rho0 if self.rho0 is not None else rho.mean()
        if abs(self._saved_rho0 - rho0) > 1e-6 or rho.shape != self._shape:
            self._kernel = wt_kernel(grid, rho0, self.x, self.alpha, self.beta)
            self._saved_rho0, self._shape = rho0, rho.shape
        return self._kernel

    def __call__(self, rho, grid, calc=("E", "V")):
        K = self.kernel(rho, grid)
        a, b = self.alpha, self.beta
        rhoc = rho.copy()
        rhoc[rho < ZERO] = ZERO                     # wt.py:15-18 (clamp, restored after)
        out = {}
        if abs(b - a) < 1e-9:
            rb = rhoc ** b
            pot = 2.0 * a * (rb / rhoc) * ifft(fft(rb, grid) * K, grid)   # wt.py:19-23
            if "V" in calc:
                out["V"] = pot
            if "E" in calc:
                if "V" in calc:
                    ed = pot * rho / (2 * a)                              # wt.py:124-125
                else:
                    ed = ifft(fft(rb, grid) * K, grid) * rb               # wt.py:44-56
                out["E"] = ed.sum() * grid.dV
        else:
            ra, rb = rhoc ** a, rhoc ** b
            if "V" in calc:
                pot = a * rhoc ** (a - 1.0) * ifft(fft(rb, grid) * K, grid)
                pot += b * rhoc ** (b - 1.0) * ifft(fft(ra, grid) * K, grid)
                out["V"] = pot
            if "E" in calc:
                out["E"] = (ifft(fft(rb, grid) * K, grid) * ra).sum() * grid.dV
        return out


# --------------------------------------------------------------------------
# Wang-Govind-Carter two-body kernel (no reference implementation: restated
# from Y. A. Wang, N. Govind, E. A. Carter, Phys. Rev. B 60, 16350 (1999);
# parity unpinned)
# --------------------------------------------------------------------------
def lindhard_d2(eta, lbda, mu, tol=1e-10):
    """F, eta F' and eta^2 F'' of the inverse Lindhard function, with the
    branch order of ``lindhard`` (kernel.py:26-35): the closed form, eta < tol,
    |eta - 1| < tol (eta F' = 48 as LindhardDerivative caps it, eta^2 F'' = 0)
    and the large-eta series above 3.65, differentiated term by term."""
    eta = np.asarray(eta, dtype=np.float64)
    tol2 = tol / 10
    F = eta.copy()
    d1 = np.zeros_like(eta)
    d2 = np.zeros_like(eta)
    c0 = (eta > tol2) & (np.abs(eta - 1.0) > tol2)
    e = eta[c0]
    A = np.log((1.0 + e) / np.abs(1.0 - e))
    e2 = e * e
    L = 0.5 + 0.25 * (1.0 - e2) * A / e
    L1 = -(1.0 + e2) * A / (4.0 * e2) + 0.5 / e
    L2 = A / (2.0 * e2 * e) - 1.0 / (e2 * (1.0 - e2))
    F[c0] = 1.0 / L - 3.0 * mu * e2 - lbda
    d1[c0] = e * (-L1 / L ** 2 - 6.0 * mu * e)
    d2[c0] = e2 * (-L2 / L ** 2 + 2.0 * L1 ** 2 / L ** 3 - 6.0 * mu)
    c1 = eta < tol
    e = eta[c1]
    sl = 1.0 / 3.0 - 3.0 * mu
    F[c1] = 1.0 - lbda + e ** 2 * sl
    d1[c1] = 2.0 * e ** 2 * sl
    d2[c1] = 2.0 * e ** 2 * sl
    c2 = np.abs(eta - 1.0) < tol
    e = eta[c2]
    F[c2] = 2.0 - lbda - 3.0 * mu + 20.0 * (e - 1.0)
    d1[c2] = 48.0 * e
    d2[c2] = 0.0
    c3 = eta > 3.65
    e = eta[c3]
    inv2 = 1.0 / e ** 2
    f = np.zeros_like(e)
    g1 = np.zeros_like(e)
    g2 = np.zeros_like(e)
    pw = inv2.copy()
    for k, coef in enumerate(_LARGE):
        m = 2.0 * (k + 1)
        f += coef * pw
        g1 += -m * coef * pw
        g2 += m * (m + 1.0) * coef * pw
        pw = pw * inv2
    F[c3] = 3.0 * (1.0 - mu) * e ** 2 - lbda - 0.6 + f
    d1[c3] = 6.0 * (1.0 - mu) * e ** 2 + g1
    d2[c3] = 6.0 * (1.0 - mu) * e ** 2 + g2
    return F, d1, d2


def wgc_taylor(gamma):
    """Coefficients of xi/k* - 1 = (t + t')/6 + c1 (t^2 + t'^2) + c2 (t + t')^2 + O(t^3)
    for xi = ((k^gamma + k'^gamma)/2)^(1/gamma), k = k*(1 + t)^(1/3)."""
    return (gamma / 3.0 - 1.0) / 12.0, (1.0 - gamma) / 72.0


def wgc_kernels(grid, rho0, x=1.0, alpha=(5 + 5 ** 0.5) / 6, beta=(5 - 5 ** 0.5) / 6, gamma=2.7):
    """K0, Ka, Kb, Kc on the half grid: the Wang-Teter kernel K(q; k) =
    c (k/k*)^p F(q/2k; x, 1) (kernel.py:325-334) with its first and second
    logarithmic derivatives in k at k* = (3 pi^2 rho0)^(1/3), combined with the
    Taylor coefficients of xi_gamma; zero at G = 0."""
    tkf = 2.0 * (3.0 * rho0 * np.pi ** 2) ** (1.0 / 3.0)
    cTF = 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
    c = 5.0 / (9.0 * alpha * beta * rho0 ** (alpha + beta - 5.0 / 3.0)) * cTF
    p = 5.0 - 3.0 * (alpha + beta)
    F, d1, d2 = lindhard_d2(grid.q / tkf, x, 1.0)
    K0 = c * F
    K1 = c * (p * F - d1)
    K2 = c * (p * (p - 1.0) * F + (2.0 - 2.0 * p) * d1 + d2)
    c1, c2 = wgc_taylor(gamma)
    Ka = K1 / 6.0
    Kb = (c1 + c2) * K1 + K2 / 72.0
    Kc = 2.0 * c2 * K1 + 2.0 / 72.0 * K2
    out = [K0, Ka, Kb, Kc]
    for k in out:
        k.flat[0] = 0.0
    return out


class WGC:
    """Nonlocal part of the WGC functional, second order in theta = (rho - rho0)/rho0:
    E = int a0 P0 + a1 P1 + a2 P2 with a_n = rho^alpha theta^n, b_n = rho^beta theta^n,
    P0 = K0*b0 + Ka*b1 + Kb*b2, P1 = Ka*b0 + Kc*b1, P2 = Kb*b0; V = sum a_n' P_n +
    b_n' Q_n (Q: the same convolutions of the a_n), rho0 held fixed (as in wt.py)."""

    def __init__(self, x=1.0, alpha=(5 + 5 ** 0.5) / 6, beta=(5 - 5 ** 0.5) / 6, gamma=2.7, rho0=None):
        self.x, self.alpha, self.beta, self.gamma, self.rho0 = x, alpha, beta, gamma, rho0

    def __call__(self, rho, grid, calc=("E", "V")):
        rho0 = self.rho0 if self.rho0 is not None else rho.mean()
        K0, Ka, Kb, Kc = wgc_kernels(grid, rho0, self.x, self.alpha, self.beta, self.gamma)
        a, b = self.alpha, self.beta
        rc = np.where(rho < ZERO, ZERO, rho)
        th = (rho - rho0) / rho0
        ra, rb = rc ** a, rc ** b
        A = [fft(ra * th ** n, grid) for n in range(3)]
        B = [fft(rb * th ** n, grid) for n in range(3)]
        P = [ifft(K0 * B[0] + Ka * B[1] + Kb * B[2], grid), ifft(Ka * B[0] + Kc * B[1], grid), ifft(Kb * B[0], grid)]
        out = {}
        if "E" in calc:
            out["E"] = (ra * (P[0] + th * (P[1] + th * P[2]))).sum() * grid.dV
        if "V" in calc:
            Q = [ifft(K0 * A[0] + Ka * A[1] + Kb * A[2], grid), ifft(Ka * A[0] + Kc * A[1], grid),
                 ifft(Kb * A[0], grid)]
            va = a * ra / rc * (P[0] + th * (P[1] + th * P[2])) + ra / rho0 * (P[1] + 2.0 * th * P[2])
            vb = b * rb / rc * (Q[0] + th * (Q[1] + th * Q[2])) + rb / rho0 * (Q[1] + 2.0 * th * Q[2])
            out["V"] = va + vb
        return out


# --------------------------------------------------------------------------
# density-dependent kernel (LWT family; the "WGC table" workload)
# --------------------------------------------------------------------------
def wt_kernel_table(eta, x=1.0):
    """WTKernelTable (kernel.py:344-352): F(eta; x, 1) * (4/5) C_TF, alpha/beta ignored."""
    factor = 4.0 / 5.0 * 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
    return lindhard(eta, x, 1.0) * factor


def mgp_kernel_table(eta, maxpoints=1000, symmetrization=None):
    """MGPKernelTable (kedf/kernel.py:267-322), serial: the MGP kernel as a sum
    over t = i/maxpoints of F(eta t^-1/3; 1, 1) / t^(1/6) (t^(-2/3) for the
    geometric symmetrisation), F from a cubic spline on a log grid evaluated
    with constant extension (splev ext=3); 'Arithmetic' averages with the WT
    table, 'Geometric' doubles."""
    dt = 1.0 / maxpoints
    cTF = 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
    coe = 4.0 / 5.0 * cTF * 5.0 / 6.0 * dt
    gp = np.logspace(np.log10(eta[1] / 10), np.log10(eta[-1] + 2), num=eta.size)
    tck = splrep(gp, lindhard(gp, 1.0, 1.0))
    kernel = np.zeros_like(eta)
    for i in range(1, maxpoints + 1):
        t = i * dt
        Gt = splev(eta / np.cbrt(t), tck, ext=3)
        t16 = t ** (-2.0 / 3.0) if symmetrization == "Geometric" else t ** (1.0 / 6.0)
        kernel += Gt / t16
    if symmetrization == "Arithmetic":
        return 0.5 * (kernel * coe + wt_kernel_table(eta))
    if symmetrization == "Geometric":
        return kernel * 2.0 * coe
    return kernel * coe


def kernel_kf(q, kf, tck, etamax):
    """LWTKernelKf (kernel.py:379-405) for a spline table: splev(q/kf) below etamax,
    the value at etamax above it, element [0,0,0] zeroed when q there is 0."""
    eta = q / kf
    K = np.empty_like(q)
    c0 = eta < etamax
    limit = splev(etamax, tck)
    if c0.any():
        K[c0] = splev(eta[c0], tck)
    K[~c0] = limit
    if q[0, 0, 0] < ZERO:
        K[0, 0, 0] = 0.0
    return K


def guess_kf_bound(kf_l, kf_r, saved, kfmin=None, kfmax=None, kftol=1e-3):
    """kedf/lwt.py:36-79 (with the persistent kfmin/kfmax state in ``saved``)."""
    kfmin_prev = saved.get("kfmin")
    kfmax_prev = saved.get("kfmax")
    if kfmin is not None and kfmax is not None:
        return [kfmin, kfmax]
    if kfmin_prev is None:
        kfmin_prev = 10
        if kfmin is None:
            kfmin = kf_l
    if kfmax_prev is None:
        kfmax_prev = 1.0
        if kfmax is None:
            kfmax = kf_r
    if kfmin is None or kfmin > kfmin_prev:
        kfmin = kfmin_prev
    if kfmax is None or kfmax < kfmax_prev:
        kfmax = kfmax_prev
    if kfmin > kf_l:
        kfl = [1e-5, 1e-4, 5e-3, 1e-3, 5e-3, 1e-2, 5e-2, 0.1, 0.5, 1.0]
        ratio = kf_l / kfmin
        for i in range(len(kfl) - 1, 0, -1):
            if ratio > kfl[i]:
                kfmin *= kfl[i]
                break
    if kfmin < kftol:
        kfmin = kftol
    if kfmax < kf_r:
        dk = kf_r - kfmax
        kfmax += (np.round(dk / 0.5) + 1) * 0.5
    saved["kfmin"] = kfmin
    saved["kfmax"] = kfmax
    return [kfmin, kfmax]


def node_list(kfMin, kfMax, nsp=None, delta=None, ratio=1.15):
    """Reference k_F nodes (lwt.py:174-190)."""
    if nsp is not None:
        if kfMax - kfMin < 1e-3:
            kfl = np.asarray([kfMin, kfMax], dtype=np.float64)
        else:
            kfl = kfMin + (kfMax - kfMin) / (nsp - 1) * np.arange(nsp)
    elif delta is not None:
        n = int(np.ceil((kfMax - kfMin) / delta)) + 1
        kfl = np.linspace(kfMin, kfMax, n)
    else:
        n = int(np.ceil(np.log(kfMax / kfMin) / np.log(ratio))) + 1
        kfl = kfMin * ratio ** np.arange(n)
    kfl = np.array(kfl, dtype=np.float64)
    kfl[0] -= 1e-16
    kfl[-1] += 1e-16
    return kfl


class LWT:
    """Density-dependent nonlocal kernel by k_F-node interpolation
    (kedf/lwt.py:502-568 table build, :82-341 potential and energy).

    The interval loop, the node arithmetic and the membership tests follow the
    reference exactly (including its quirks: points exactly at the first/last
    node belong to no interval; the first node has a 'small-k_F' branch).
    ``interp`` is 'linear' or 'hermite'.  MGP lump factors are not supported.
    """

    def __init__(self, x=1.0, alpha=5.0 / 6.0, beta=5.0 / 6.0, etamax=50.0, neta=50000,
                 order=3, interp="linear", kdd=3, ratio=1.15, nsp=None, delta=None,
                 kfmin=None, kfmax=None, ldw=None, kerneltype="WT", symmetrization=None, maxpoints=1000):
        self.x, self.alpha, self.beta = x, alpha, beta
        self.kerneltype, self.symmetrization, self.maxpoints = kerneltype, symmetrization, maxpoints
        self.etamax, self.neta, self.order = etamax, neta, order
        self.interp, self.kdd, self.ratio, self.nsp, self.delta = interp, kdd, ratio, nsp, delta
        self.kfmin, self.kfmax, self.ldw = kfmin, kfmax, ldw
        self.saved = {"kfmin": None, "kfmax": None, "shape": None}
        self.tables()

    def tables(self):
        """lwt.py:535-566 (order 3): the WT table or an MGP table (kerneltype
        'MGP' with its symmetrisation, 'MGPA' arithmetic, 'MGPG' geometric)."""
        eta = np.linspace(0, self.etamax, self.neta)
        if self.kerneltype == "WT":
            table = wt_kernel_table(eta, self.x)
        else:
            sym = {"MGP": self.symmetrization, "MGPA": "Arithmetic", "MGPG": "Geometric"}[self.kerneltype]
            table = mgp_kernel_table(eta, self.maxpoints, sym)
        self.tck = splrep(eta, table, k=self.order)
        deriv = splev(eta, self.tck, der=1) * (-1.0 * eta)
        self.tckD = splrep(eta, deriv, k=self.order)

    def timed_sample(self, rho, grid, intervals=1):
        """Wall time of one E+V split into the part outside the node-interval loop
        and the mean time of one interval, running only ``intervals`` of them
        (a bounded sample of a full evaluation for CPU baselines)."""
        import time
        timing = {}
        t0 = time.perf_counter()
        self(rho, grid, ("E", "V"), max_intervals=intervals, timing=timing)
        total = time.perf_counter() - t0
        loop = timing.get("loop", 0.0)
        n = max(1, timing.get("intervals", 1))
        return total - loop, loop / n

    def __call__(self, rho, grid, calc=("E", "V"), max_intervals=None, timing=None):
        """LWTPotentialEnergy (lwt.py:82-341), streamed interval by interval like the
        reference so that memory stays O(grid).  ``max_intervals``/``timing`` only
        serve timed samples (the result is then incomplete)."""
        alpha, beta = self.alpha, self.beta
        q = grid.q
        kf = 2.0 * np.cbrt(3.0 * np.pi ** 2 * rho)                     # lwt.py:106
        out = {}
        if abs(kf.max() - kf.min()) < 1e-8:                           # lwt.py:115-124 (HEG)
            if "E" in calc:
                out["E"] = 0.0
            if "V" in calc:
                out["V"] = np.zeros_like(rho)
            return out
        kfb = guess_kf_bound(kf.min(), kf.max(), self.saved, self.kfmin, self.kfmax)
        vcalc = "V" in calc
        kdd = self.kdd if vcalc else 1
        if (kf > kfb[1]).any():                                       # lwt.py:145-146
            kf = np.minimum(kf, kfb[1])
        kfMin = max(kf.min(), kfb[0]) if self.kfmin is None else self.kfmin
        kfMax = kf.max() if self.kfmax is None else self.kfmax
        kfl = node_list(kfMin, kfMax, self.nsp, self.delta, self.ratio)
        nsp = len(kfl)
        rhoc = rho.copy()                                             # lwt.py:206-221
        rhoc[~(rho > 0)] = 1e-30
        rA = rhoc ** alpha
        rA1 = rA / rhoc
        if abs(alpha - beta) < 1e-8:
            rB, rB1 = rA, rA1
        else:
            rB = rhoc ** beta
            rB1 = rB / rhoc
        rBG = fft(rB, grid)
        hermite = self.interp == "hermite"
        mcalc = kdd > 1 or hermite
        pot1 = np.zeros_like(rho)
        pot3 = np.zeros_like(rho)
        pot2G = None

        def node(j):
            K = kernel_kf(q, kfl[j], self.tck, self.etamax)
            p = ifft(K * rBG, grid)
            if mcalc:
                KD = kernel_kf(q, kfl[j], self.tckD, self.etamax) / kfl[j]
                return K, p, KD, ifft(KD * rBG, grid)
            return K, p, None, None

        K0, p0, KD0, m0 = node(0)
        small = kf < kfl[0] + 1e-18                                   # lwt.py:254-266
        t = (kf - kfl[0]) / kfl[0]
        pot1[small] = p0[small] * t[small]
        if kdd > 1:
            pot2G = K0 * fft(rA * np.where(small, t, 0.0), grid)
        import time as _time
        _tl = _time.perf_counter()
        n_run = nsp - 1 if max_intervals is None else min(nsp - 1, max_intervals)
        for i in range(n_run):                                        # lwt.py:213-306
            K1, p1, KD1, m1 = node(i + 1)
            m = np.logical_and(kf > kfl[i], kf < kfl[i + 1] + 1e-18)
            u = np.where(m, rA, 0.0)
            Dkf = kfl[i + 1] - kfl[i]
            t = (kf - kfl[i]) / Dkf
            if not hermite:
                t0 = 1 - t
                pot1[m] = p0[m] * t0[m] + p1[m] * t[m]
                if kdd > 1:
                    pot2G = pot2G + K0 * fft(u * t0, grid) + K1 * fft(u * t, grid)
                    if kdd == 3:
                        pot3[m] = m0[m] * t0[m] + m1[m] * t[m]
            else:
                t2 = t * t
                t3 = t2 * t
                h00 = 2.0 * t3 - 3.0 * t2 + 1.0
                h10 = t3 - 2.0 * t2 + t
                h01 = 1.0 - h00
                h11 = t3 - t2
                pot1[m] = h00[m] * p0[m] + h01[m] * p1[m] + Dkf * (h10[m] * m0[m] + h11[m] * m1[m])
                if kdd > 1:
                    pot2G = pot2G + (K0 * fft(u * h00, grid) + K1 * fft(u * h01, grid)
                                     + Dkf * (KD0 * fft(u * h10, grid) + KD1 * fft(u * h11, grid)))
                    if kdd == 3:
                        tm, t2m = t[m], t2[m]
                        h00D = 6.0 * t2m - 6 * tm
                        h10D = 3.0 * t2m - 4 * tm + 1.0
                        h01D = -h00D
                        h11D = 3.0 * t2m - 2 * tm
                        pot3[m] = (h00D * p0[m] + h01D * p1[m]) / Dkf + h10D * m0[m] + h11D * m1[m]
            K0, p0, KD0, m0 = K1, p1, KD1, m1
        if timing is not None:
            timing["loop"] = _time.perf_counter() - _tl
            timing["intervals"] = n_run
        if vcalc:
            pot2 = ifft(pot2G, grid) if pot2G is not None else pot1.copy()
        ldw = 1.0 / 6.0 if self.ldw is None else self.ldw            # lwt.py:315-322
        factor = np.ones_like(rho)
        rhov = rho.max()
        lm = rho < 1e-6
        ld = max(0.1, ldw)
        factor[lm] = np.abs(rho[lm]) ** ld / (rhov ** ld)
        factor[rho < 0] = 0.0
        pot1 = pot1 * factor
        if "E" in calc:
            out["E"] = (rA * pot1).sum() * grid.dV                    # lwt.py:326-327
        if vcalc:
            pot2 = pot2 * factor
            pot3 = pot3 * factor
            out["V"] = alpha * rA1 * pot1 + beta * rB1 * pot2 + (kf / 3.0) * rA1 * pot3
        return out



# --------------------------------------------------------------------------
# HC / revHC (kedf/hc.py:16-439, kernel.py:460-506)
# --------------------------------------------------------------------------
def hc_kernel_table(eta, beta=2.0 / 3.0, x=1.0):
    """HCKernelTable (kernel.py:460-478): the ODE beta eta K' = -5/3 F(eta; x, 1) +
    (5 - 3 beta) beta K integrated by scipy's odeint from eta[-1] (K = -8/3 /
    ((5 - 3 beta) beta)) down to 0, K[0] = 0, times C_TF 8 (3 pi^2)."""
    from scipy.integrate import odeint

    def lind_scalar(e, lbda, mu, tol=1e-10):
        # LindhardFunction on a Python float (kernel.py:36-44): the first true
        # branch wins, so above eta = 3.65 the closed form is used, not the series
        tol2 = tol / 10
        if e > tol2 and abs(e - 1.0) > tol2:
            return 1.0 / (0.5 + 0.25 * (1.0 - e ** 2) * np.log((1.0 + e) / np.abs(1.0 - e)) / e) - 3.0 * mu * e ** 2 - lbda
        if e < tol:
            return 1.0 - lbda + e ** 2 * (1.0 / 3.0 - 3.0 * mu)
        if abs(e - 1.0) < tol:
            return 2.0 - lbda - 3.0 * mu + 20.0 * (e - 1.0)
        return float(lindhard(np.array([e]), lbda, mu)[0])

    def deriv(k, e):  # hc_ode_deriv (kernel.py:481-492), e a float as odeint passes it
        d = -5.0 / 3.0 * lind_scalar(e, x, 1) + (5.0 - 3.0 * beta) * beta * k
        if e > 1e-20:
            d /= beta * e
        return d

    k_inf = -8.0 / 3.0 / ((5.0 - 3.0 * beta) * beta)
    sol = odeint(deriv, k_inf, eta[::-1])
    kernel = sol.ravel()[::-1].copy()
    kernel[0] = 0.0
    return kernel * (3.0 / 10.0) * (3.0 * np.pi ** 2) ** (2.0 / 3.0) * 8.0 * 3.0 * np.pi ** 2


def hc_kflist(kf_min, kf_max, saved, kf0=1.0, ratio=1.15, nsp=None, delta=None, kfmin=None, kfmax=None,
              savetol=1e-16):
    """get_kflist (hc.py:16-66): bounds snapped to powers of ratio, kept from the
    saved state when they moved little, nodes by nsp, delta or ratio."""
    kfmin_prev, kfmax_prev = saved.get("kfmin"), saved.get("kfmax")
    if kfmin is None:
        kfmin = max(kf_min, 1e-3)
        n = int(np.floor(np.log(kfmin / kf0) / np.log(ratio))) - 1
        kfmin = kf0 * ratio ** n
    if kfmax is None:
        kfmax = min(kf_max, 100)
        n = int(np.ceil(np.log(kfmax / kf0) / np.log(ratio))) + 1
        kfmax = kf0 * ratio ** n
    if kfmin_prev is not None and kfmin > kfmin_prev and (kfmin - kfmin_prev) < 0.2:
        kfmin = kfmin_prev
    if kfmax_prev is not None and kfmax < kfmax_prev and (kfmax_prev - kfmax) < 1:
        kfmax = kfmax_prev
    if nsp is not None:
        if kfmax - kfmin < 1e-3:
            kfl = np.array([kfmin, kfmax], dtype=np.float64)
        else:
            kfl = kfmin + (kfmax - kfmin) / (nsp - 1) * np.arange(nsp)
    elif delta is not None:
        kfl = np.linspace(kfmin, kfmax, int(np.ceil((kfmax - kfmin) / delta)) + 1)
    else:
        kfl = kfmin * ratio ** np.arange(int(np.log(kfmax / kfmin) / np.log(ratio)) + 1)
    kfl = np.asarray(kfl, dtype=np.float64)
    kfl[0] -= savetol
    kfl[-1] += savetol
    saved["kfmin"], saved["kfmax"] = kfmin, kfmax
    return kfl


def _ggafs_hc(s, functional, params):
    """The enhancement factors HC and revHC use (hc.py:115-131, GGAFs gga.py:653-1210):
    'HC' F = 1 + lambda s^2; 'PBE2' F = 1 + p1 ss^2 / (1 + p0 ss^2), ss = s / TKF0."""
    f = functional.upper()
    if f == "HC":
        lam = 0.0 if params is None else params[0]
        return 1 + lam * s * s, 2 * lam * np.ones_like(s)
    if f == "PBE2":
        p = [2.0309 / 0.2942, 2.0309] if params is None else list(params)
        ss = s / TKF0
        s2 = ss * ss
        Fb = 1.0 + p[0] * s2
        return 1.0 + p[1] * s2 / Fb, 2.0 * p[1] / (Fb * Fb) / (TKF0 * TKF0)
    raise NotImplementedError(functional)


class HC:
    """HC / revHC (hc.py:68-439) with Hermite interpolation between nodes."""

    def __init__(self, alpha=2.0, beta=2.0 / 3.0, x=1.0, etamax=50.0, neta=50000, ratio=1.15, nsp=None,
                 delta=None, kfmin=None, kfmax=None, ldw=None, functional="HC", params=None):
        self.alpha, self.beta, self.etamax = alpha, beta, etamax
        self.ratio, self.nsp, self.delta, self.kfmin, self.kfmax, self.ldw = ratio, nsp, delta, kfmin, kfmax, ldw
        self.functional, self.params = functional, params
        eta = np.linspace(0, etamax, neta)
        table = hc_kernel_table(eta, beta=beta, x=x)
        self.tck = splrep(eta, table, k=3)
        self.tckD = splrep(eta, splev(eta, self.tck, der=1) * (-1.0 * eta), k=3)
        self.saved = {"kfmin": None, "kfmax": None}

    def _xi(self, q, k):
        """HCKernelXi (kernel.py:496-506): xi = 2k, K = T(q/xi)/xi^3, K' = (TD - 3T)/xi^3."""
        xi = 2.0 * k
        T = kernel_kf(q, xi, self.tck, self.etamax)
        TD = kernel_kf(q, xi, self.tckD, self.etamax)
        return T / xi ** 3, (TD - 3 * T) / xi ** 3

    def __call__(self, rho_in, grid, calc=("E", "V")):
        alpha, beta = self.alpha, self.beta
        rho = rho_in.copy()
        rho[rho < ZERO] = ZERO                                        # hc.py:88-90
        rA = rho ** alpha
        rA1 = rA / rho
        if abs(alpha - beta) < 1e-8:
            rB, rB1 = rA, rA1
        else:
            rB = rho ** beta
            rB1 = rB / rho
        rBG = fft(rB, grid)
        rho43 = rho ** (4.0 / 3.0)
        rho83 = rho43 * rho43
        q = grid.q
        rG = fft(rho, grid)
        grad = [ifft(grid.g[i] * rG * 1j, grid) for i in range(3)]
        s = np.sqrt(grad[0] ** 2 + grad[1] ** 2 + grad[2] ** 2) / rho43
        F, dFds2 = _ggafs_hc(s, self.functional, self.params)
        kf_std = np.cbrt(3.0 * np.pi ** 2 * rho)
        kf = F * kf_std
        kfl = hc_kflist(kf.min(), kf.max(), self.saved, 1.0, self.ratio, self.nsp, self.delta, self.kfmin,
                        self.kfmax)
        nsp = len(kfl)
        out = {}
        if abs(kf.max() - kf.min()) < 1e-8 or nsp < 3:              # hc.py:150-158 (HEG)
            out["E"] = 0.0
            out["V"] = np.zeros_like(rho)
            return out
        kf = np.where(kf > kfl[-1], kfl[-1], kf)
        pot1 = np.zeros_like(rho)
        pot3 = np.zeros_like(rho)

        def node(j):
            K, KD = self._xi(q, kfl[j])
            KD = KD / kfl[j]
            return K, ifft(K * rBG, grid), KD, ifft(KD * rBG, grid)

        K0, p0, KD0, m0 = node(0)
        small = kf < kfl[0] + 1e-18                                   # hc.py:203-215
        t = (kf - kfl[0]) / kfl[0]
        pot1[small] = p0[small] * t[small]
        pot2G = K0 * fft(rA * np.where(small, t, 0.0), grid)
        for i in range(nsp - 1):
            K1, p1, KD1, m1 = node(i + 1)
            m = np.logical_and(kf > kfl[i], kf < kfl[i + 1] + 1e-18)
            u = np.where(m, rA, 0.0)
            Dkf = kfl[i + 1] - kfl[i]
            t = (kf - kfl[i]) / Dkf
            t2 = t * t
            t3 = t2 * t
            h00 = 2.0 * t3 - 3.0 * t2 + 1.0
            h10 = t3 - 2.0 * t2 + t
            h01 = 1.0 - h00
            h11 = t3 - t2
            pot1[m] = h00[m] * p0[m] + h01[m] * p1[m] + Dkf * (h10[m] * m0[m] + h11[m] * m1[m])
            pot2G = pot2G + (K0 * fft(u * h00, grid) + K1 * fft(u * h01, grid)
                             + Dkf * (KD0 * fft(u * h10, grid) + KD1 * fft(u * h11, grid)))
            tm, t2m = t[m], t2[m]
            h00D = 6.0 * t2m - 6 * tm
            h10D = 3.0 * t2m - 4 * tm + 1.0
            h01D = -h00D
            h11D = 3.0 * t2m - 2 * tm
            pot3[m] = (h00D * p0[m] + h01D * p1[m]) / Dkf + h10D * m0[m] + h11D * m1[m]
            K0, p0, KD0, m0 = K1, p1, KD1, m1
        pot2 = ifft(pot2G, grid)
        out["E"] = (rA * pot1).sum() * grid.dV                         # hc.py:294-297
        if "V" in calc:                                               # hc.py:301-331
            pot1 = pot1 * alpha * rA1
            pot2 = pot2 * beta * rB1
            pot3 = pot3 * rA
            pot3_1 = kf_std / (3 * rho) * (F - 4 * dFds2 * s * s) * pot3
            pot_dn = kf_std * dFds2 / rho83 * pot3
            p3 = [fft(grad[i] * pot_dn, grid) for i in range(3)]
            pot3G = grid.g[0] * p3[0] + grid.g[1] * p3[1] + grid.g[2] * p3[2]
            pot3_2 = ifft(1j * pot3G, grid)
            pot = pot1 + pot2 + pot3_1 - pot3_2
            ldw = 1.0 / 6.0 if self.ldw is None else self.ldw
            factor = np.ones_like(rho)
            rhov = rho.max()
            lm = rho < 1e-6
            ld = max(0.1, ldw)
            factor[lm] = np.abs(rho[lm]) ** ld / (rhov ** ld)
            factor[rho < 0] = 0.0
            out["V"] = pot * factor
        return out


# --------------------------------------------------------------------------
# pseudopotential: recpot I/O, radial lines, PME structure factor
# --------------------------------------------------------------------------
def write_recpot(fname, gmax_bohr_inv, v_ha_bohr3, header="synthetic"):
    """CASTEP .recpot writer (format of functional/pseudo/recpot.py:11-42): eV*A^3 on a
    uniform G grid from 0 to gmax (A^-1), three values per line, terminator '1000'."""
    v = np.asarray(v_ha_bohr3) * HARTREE * BOHR ** 3
    gmax = gmax_bohr_inv / BOHR
    lines = ["START COMMENT", header, "END COMMENT", "3     5", repr(float(gmax))]
    for i in range(0, len(v), 3):
        lines.append("  ".join("%.17e" % x for x in v[i:i + 3]))
    lines.append("1000")
    with open(fname, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_recpot(fname):
    """recpot.py:11-42: returns (gp [Bohr^-1], vp [Ha Bohr^3], zval)."""
    with open(fname) as f:
        lines = f.readlines()
    ibegin = 0
    iend = None
    for i, line in enumerate(lines):
        if "END COMMENT" in line:
            ibegin = i + 3
        elif ibegin > 1 and (line.strip() == "1000" or len(line.strip()) == 1):
            iend = i
            break
    vals = " ".join(l.strip() for l in lines[ibegin:iend]).split()
    gmax = float(lines[ibegin - 1].strip()) * BOHR
    v = np.array(vals, dtype=np.float64) / HARTREE / BOHR ** 3
    r = np.linspace(0, gmax, num=len(v))
    zval = round((v[0] - v[1]) * (r[1] ** 2) / (4.0 * np.pi))
    return r, v, zval


def synthetic_pp(Z, rc, A=15.0, npts=4096, gmax=40.0):
    """v(G) = -4 pi Z/G^2 exp(-G^2 rc^2/4) + A exp(-G^2 rc^2/4), G=0 limit A + pi Z rc^2."""
    g = np.linspace(0.0, gmax, npts)
    v = np.empty_like(g)
    e = np.exp(-g[1:] ** 2 * rc ** 2 / 4.0)
    v[1:] = -4.0 * np.pi * Z / g[1:] ** 2 * e + A * e
    v[0] = A + np.pi * Z * rc ** 2
    return g, v


def quartic(f, dx):
    """math_utils.quartic_interpolation (math_utils.py:390-400)."""
    t0 = f[2]
    t1 = 2.0 * f[0] - 16.0 * f[1] + 16.0 * f[3] - 2.0 * f[4]
    t2 = -f[0] + 16.0 * f[1] - 30.0 * f[2] + 16.0 * f[3] - f[4]
    t3 = -2.0 * f[0] + 4.0 * f[1] - 4.0 * f[3] + 2.0 * f[4]
    t4 = f[0] - 4.0 * f[1] + 6.0 * f[2] - 4.0 * f[3] + f[4]
    return t0 + dx * (t1 + dx * (t2 + dx * (t3 + dx * t4))) / 24.0


def vline(grid, gp, vp):
    """LocalPseudo.calc_vlines (pseudo/__init__.py:398-423) with the spline of
    ReadPseudo.get_vloc_interp (:689-706): splrep(gp[1:], vp[1:], k=3)."""
    tck = splrep(gp[1:], vp[1:], k=3)
    q = grid.q
    out = np.zeros_like(q)
    m = q < gp[-1]
    if m.any():
        out[m] = splev(q[m], tck, der=0)
    m = q < gp[1]
    dp = gp[1] - gp[0]
    out[m] = quartic([vp[2], vp[1], vp[0], vp[1], vp[2]], q[m] / dp)
    return out


def bspline_Mn(x, order):
    """CBspline.calc_Mn (ewald.py:63-82): Mn[n] = M_order(x + n - 1), n = 1..order."""
    Mn = np.zeros(order + 1)
    Mn[1] = x
    Mn[2] = 1.0 - x
    for i in range(3, order + 1):
        for j in range(0, i):
            n = i - j
            Mn[n] = (x + n - 1) * Mn[n] + (j + 1 - x) * Mn[n - 1]
            Mn[n] /= i - 1
    return Mn


def bspline_Mn_full(x, order_full, order):
    """calc_Mn(x, order) of an object built for ``order_full`` (array length order_full+1)."""
    Mn = np.zeros(order_full + 1)
    Mn[1] = x
    Mn[2] = 1.0 - x
    for i in range(3, order + 1):
        for j in range(0, i):
            n = i - j
            Mn[n] = (x + n - 1) * Mn[n] + (j + 1 - x) * Mn[n - 1]
            Mn[n] /= i - 1
    return Mn


def bspline_barray(grid, order=10):
    """CBspline._calc_bm + Barray (ewald.py:44-55, :84-101)."""
    Mn = bspline_Mn(1.0, order)
    bm = []
    for d in range(3):
        qd = 2.0 * np.pi * np.arange(grid.nrG[d]) / grid.nr[d]
        tmp = np.exp(-1j * (order - 1.0) * qd)
        fac = np.zeros_like(tmp)
        for k in range(1, order):
            fac += Mn[k] * np.exp(-1j * k * qd)
        bm.append(tmp / fac)
    return np.einsum("i,j,k->ijk", bm[0], bm[1], bm[2])


def scaled_positions(pos, lattice):
    """ase get_scaled_positions(wrap=True): fractional coordinates wrapped to [0,1)."""
    fr = np.linalg.solve(np.asarray(lattice).T, np.asarray(pos, dtype=np.float64).T).T
    fr = fr % 1.0
    fr[fr == 1.0] = 0.0
    return fr


def pme_qarray(grid, frac, weights, order=10):
    """CBspline.get_PME_Qarray / _calc_PME_Qarray (ewald.py:137-194): spread each atom's
    order^3 B-spline stencil (indices mod n) with weight ``weights[a]``."""
    Q = np.zeros(tuple(grid.nr))
    ix = np.arange(order)
    for a in range(len(frac)):
        Up = frac[a] * grid.nr
        fl = np.floor(Up).astype(np.int64)
        Mn = [bspline_Mn(Up[d] - np.floor(Up[d]), order)[1:] for d in range(3)]
        l = [np.mod(1 + fl[d] - ix, grid.nr[d]) for d in range(3)]
        val = weights[a] * np.einsum("i,j,k->ijk", Mn[0], Mn[1], Mn[2])
        # each stencil point is distinct for n >= order, so plain fancy += is exact
        Q[np.ix_(l[0], l[1], l[2])] += val
    return Q


class LocalPseudo:
    """LocalPseudo (pseudo/__init__.py:74-452, :505-571): v_loc on the grid by PME
    (B-spline structure factor) or by the exact structure factor."""

    def __init__(self, grid, pos, species, tables, PME=True, order=10):
        """tables: list of (gp, vp) per species index; species: int array per atom."""
        self.grid, self.PME, self.order = grid, PME, order
        self.pos = np.asarray(pos, dtype=np.float64)
        self.species = np.asarray(species)
        self.tables = tables
        self.vlines = [vline(grid, gp, vp) for gp, vp in tables]
        self._vreal = None

    @property
    def vreal(self):
        if self._vreal is None:
            g = self.grid
            v = np.zeros(tuple(g.nrG), dtype=np.complex128)
            if self.PME:          # _PP_Reciprocal_PME (:437-452)
                frac = scaled_positions(self.pos, g.lattice)
                for s in range(len(self.tables)):
                    sel = self.species == s
                    Q = pme_qarray(g, frac[sel], np.ones(sel.sum()), self.order)
                    v = v + self.vlines[s] * fft(Q, g)
                v = v * bspline_barray(g, self.order) * g.nnr / g.volume
            else:                 # _PP_Reciprocal (:425-435)
                gv = g.g
                for s in range(len(self.tables)):
                    for a in np.nonzero(self.species == s)[0]:
                        strf = np.exp(-1j * np.einsum("lijk,l->ijk", gv, self.pos[a]))
                        v += self.vlines[s] * strf
            self._vreal = ifft(v, g)
        return self._vreal

    def __call__(self, rho, calc=("E", "V")):
        out = {"V": self.vreal}
        if "E" in calc:
            out["E"] = np.einsum("ijk,ijk->", self.vreal, rho) * self.grid.dV
        return out

    def forces(self, rho):
        g = self.grid
        rhoG = fft(rho, g)
        nat = len(self.pos)
        F = np.zeros((nat, 3))
        if not self.PME:      # _Force (:505-521)
            mask = g.mask
            gv = g.g
            for a in range(nat):
                istrf = np.exp(1j * np.einsum("lijk,l->ijk", gv, self.pos[a]))
                den = self.vlines[self.species[a]][mask] * (rhoG[mask] * istrf[mask]).imag
                for j in range(3):
                    F[a, j] = np.einsum("i,i->", gv[j][mask], den)
            return F * 2.0 / g.volume
        # _ForcePME (:523-571)
        B = np.conjugate(bspline_barray(g, self.order))
        denG = rhoG * B
        cell_inv = g.rlattice.T / 2 / np.pi
        frac = scaled_positions(self.pos, g.lattice)
        o = self.order
        ix = np.arange(o)
        for s in range(len(self.tables)):
            dGV = denG * self.vlines[s]
            dGV[0, 0, 0] = 0.0
            rhoPB = ifft(dGV, g)
            for a in np.nonzero(self.species == s)[0]:
                F[a] = -_pme_gather_grad(g, frac[a], o, cell_inv, rhoPB)
        return F


def _pme_gather_grad(grid, frac, o, cell_inv, field):
    """sum over the B-spline stencil of (dQ/du . cell_inv) * field (ewald.py:846-862)."""
    Up = frac * grid.nr
    fl = np.floor(Up).astype(np.int64)
    Mn = [bspline_Mn(Up[d] - np.floor(Up[d]), o) for d in range(3)]
    M2 = [bspline_Mn_full(Up[d] - np.floor(Up[d]), o, o - 1) for d in range(3)]
    dM = [M2[d][1:] - M2[d][:-1] for d in range(3)]
    Mv = [Mn[d][1:] for d in range(3)]
    dQ = np.empty((3, o, o, o))
    dQ[0] = grid.nr[0] * np.einsum("i,j,k->ijk", dM[0], Mv[1], Mv[2])
    dQ[1] = grid.nr[1] * np.einsum("i,j,k->ijk", Mv[0], dM[1], Mv[2])
    dQ[2] = grid.nr[2] * np.einsum("i,j,k->ijk", Mv[0], Mv[1], dM[2])
    ix = np.arange(o)
    l = [np.mod(1 + fl[d] - ix, grid.nr[d]) for d in range(3)]
    fv = field[np.ix_(l[0], l[1], l[2])]
    return np.einsum("d,dk->k", np.einsum("dijk,ijk->d", dQ, fv), cell_inv)


# --------------------------------------------------------------------------
# Ewald
# --------------------------------------------------------------------------
def erfcinv(y):
    return sp.erfcinv(y)


class Ewald:
    """Ewald ion-ion energy and forces (ewald.py:197-864).  The real-space sum is the
    exact truncated image sum of Energy_real (:281-325); for orthorhombic cells the
    reference's windowed Energy_real_fast2 (:372-446) visits the same pairs."""

    def __init__(self, grid, pos, charges, precision=1e-8, PME=True, order=10):
        self.grid = grid
        self.pos = np.asarray(pos, dtype=np.float64)
        self.q = np.asarray(charges, dtype=np.float64)
        self.precision, self.PME, self.order = precision, PME, order
        gmax = np.sqrt(2.0 * grid.guess_ecut())
        self.eta = self.best_eta(precision, gmax)

    def best_eta(self, precision, gmax):
        """Get_Best_eta (ewald.py:256-278)."""
        q2 = np.sum(self.q * self.q)
        nat = len(self.q)
        eta = 1.6
        while True:
            up = 4.0 * np.pi * nat * q2 * np.sqrt(eta / np.pi) * sp.erfc(gmax / 2.0 * np.sqrt(1.0 / eta))
            if up < precision:
                return eta
            eta = eta - 0.01

    def _images(self):
        L = np.sqrt(np.einsum("ij->i", self.grid.lattice ** 2))
        rmax = erfcinv(self.precision / 3.0) / np.sqrt(self.eta)
        N = np.ceil(rmax / L).astype(np.int64)
        shifts = np.array([[ix, iy, iz] for ix in range(-N[0], N[0] + 1)
                           for iy in range(-N[1], N[1] + 1) for iz in range(-N[2], N[2] + 1)],
                          dtype=np.float64)
        return shifts @ self.grid.lattice, rmax

    def energy_real(self):
        R, Rcut = self._images()
        es = np.sqrt(self.eta)
        E = 0.0
        for i in range(len(self.pos)):
            d = self.pos[None, :, :] - R[:, None, :] - self.pos[i][None, None, :]
            d = np.sqrt((d * d).sum(-1))
            qq = np.broadcast_to(self.q[None, :], d.shape)
            m = (d < Rcut) & (d > 0.001)
            E += self.q[i] * np.sum(qq[m] * sp.erfc(es * d[m]) / d[m])
        return E / 2.0

    def energy_corr(self):
        """Energy_corr (ewald.py:468-482)."""
        dc = -np.sqrt(self.eta / np.pi) * np.sum(self.q * self.q)
        gz = -4.0 * np.pi * (1.0 / (4.0 * self.eta * self.grid.volume) / 2.0) * np.sum(self.q) ** 2
        return dc + gz

    def _qgrid(self):
        frac = scaled_positions(self.pos, self.grid.lattice)
        return pme_qarray(self.grid, frac, self.q, self.order), frac

    def energy_rec(self):
        g = self.grid
        if self.PME:      # Energy_rec_PME (:786-807)
            Q, _ = self._qgrid()
            strf = fft(Q, g) * bspline_barray(g, self.order)
            s2 = (np.conjugate(strf) * strf)
            m = g.mask
            e = np.sum(s2[m] * np.exp(-g.gg[m] / (4.0 * self.eta)) * g.invgg[m])
            return 4.0 * np.pi * e.real / g.volume / g.dV ** 2
        # Energy_rec (:449-466)
        strf = np.zeros(tuple(g.nrG), dtype=np.complex128)
        for a in range(len(self.pos)):
            strf += np.exp(-1j * np.einsum("lijk,l->ijk", g.g, self.pos[a])) * self.q[a]
        s2 = np.conjugate(strf) * strf
        m = g.mask
        e = np.sum(s2[m] * np.exp(-g.gg[m] / (4.0 * self.eta)) * g.invgg[m])
        return 4.0 * np.pi * e.real / g.volume

    def energy(self):
        return self.energy_corr() + self.energy_real() + self.energy_rec()

    def forces_real(self):
        """Forces_real (ewald.py:541-577)."""
        R, Rcut = self._images()
        es = np.sqrt(self.eta)
        F = np.zeros((len(self.pos), 3))
        for i in range(len(self.pos)):
            rj = (self.pos[None, :, :] - R[:, None, :]).reshape(-1, 3)
            qj = np.broadcast_to(self.q[None, :], (len(R), len(self.q))).ravel()
            dv = self.pos[i][None, :] - rj
            d = np.sqrt((dv * dv).sum(-1))
            m = (d < Rcut) & (d > 0.001)
            x = d[m] * es
            w = sp.erfc(x) / x ** 3 + 2.0 / np.sqrt(np.pi) * np.exp(-x ** 2) / x ** 2
            F[i] = self.q[i] * np.einsum("ij,i->j", dv[m] * qj[m][:, None], w)
        return F * es ** 3

    def forces_rec(self):
        g = self.grid
        if self.PME:      # Forces_rec_PME (:810-864)
            Q, frac = self._qgrid()
            B = bspline_barray(g, self.order)
            strf = fft(Q, g) * (B * np.conjugate(B))
            strf *= np.exp(-g.gg / (4.0 * self.eta)) * g.invgg
            conv = ifft(strf, g)
            cell_inv = np.linalg.inv(g.lattice)
            F = np.zeros((len(self.pos), 3))
            for a in range(len(self.pos)):
                F[a] = -_pme_gather_grad(g, frac[a], self.order, cell_inv, conv) * self.q[a]
            return F * 4.0 * np.pi / g.dV
        # Forces_rec (:580-607)
        strf = np.zeros(tuple(g.nrG), dtype=np.complex128)
        for a in range(len(self.pos)):
            strf += np.exp(-1j * np.einsum("lijk,l->ijk", g.g, self.pos[a])) * self.q[a]
        m = g.mask
        F = np.empty((len(self.pos), 3))
        w = np.exp(-g.gg[m] / (4.0 * self.eta)) * g.invgg[m]
        for a in range(len(self.pos)):
            s = np.exp(-1j * np.einsum("lijk,l->ijk", g.g, self.pos[a]))[m] * self.q[a]
            F[a] = np.einsum("ij,j->i", g.g[:, m], (s.real * strf.imag[m] - s.imag * strf.real[m]) * w)
        return F * 8.0 * np.pi / g.volume

    def forces(self):
        return self.forces_real() + self.forces_rec()


# --------------------------------------------------------------------------
# GGA KEDFs (kedf/gga.py:18-586 enhancement factors, :1212-1325 GGA)
# --------------------------------------------------------------------------
TKF0 = 6.18733545256027186194       # src/dftpy/constants.py:83
CBRT_TWO = 1.25992104989487316477   # src/dftpy/constants.py:84


def _power_int(x, num, den=1):
    """PowerInt (math_utils.py:158-173)."""
    y = x.copy()
    for _ in range(num - 1):
        y = y * x
    if den == 1:
        return y
    if den == 2:
        return np.sqrt(y)
    if den == 3:
        return np.cbrt(y)
    if den == 4:
        return np.sqrt(np.sqrt(y))
    return np.power(y, 1.0 / den)


def _tkf0(f):
    """s_with_tkf0 (gga.py:18-40): the formula in ss = s/TKF0, dF/ds2 rescaled."""
    def w(s, p):
        F, d = f(s / TKF0, p)
        return F, d / (TKF0 * TKF0)
    return w


@_tkf0
def _lkt_mvw(ss, p):
    e1, e2 = np.exp(-p[0] * ss), np.exp(-2.0 * p[0] * ss)
    F = 2.0 * e1 / (1.0 + e2)
    return F, -p[0] * (1.0 - e2) / (1.0 + e2) * F / ss


def _dk(s, p):
    x = s * s / (72 * C_TF)
    Fa = 9.0 * p[5] * x ** 4 + p[2] * x ** 3 + p[1] * x ** 2 + p[0] * x + 1.0
    Fb = p[5] * x ** 3 + p[4] * x ** 2 + p[3] * x + 1.0
    d = (36.0 * p[5] * x ** 3 + 3 * p[2] * x ** 2 + 2 * p[1] * x + p[0]) / Fb - Fa / (Fb * Fb) * (
        3.0 * p[5] * x ** 2 + 2.0 * p[4] * x + p[3])
    return Fa / Fb, d / (36.0 * C_TF)


def _llp(s, p):
    bs = CBRT_TWO * s
    bs2 = bs * bs
    Fa = p[0] * bs2
    Fb = 1.0 + p[1] * bs * np.arcsinh(bs)
    d = 2.0 * p[0] / Fb - (p[0] * p[1] * bs * np.arcsinh(bs) + Fa * p[1] / np.sqrt(1.0 + bs2)) / (Fb * Fb)
    return 1.0 + Fa / Fb, d * (CBRT_TWO * CBRT_TWO)


def _ol(s, p):
    F = 1.0 + s * s / 72.0 / C_TF + p[0] / C_TF * s / (1 + p[1] * 4 * s)
    d = 1.0 / 36.0 / C_TF * np.ones_like(s)
    m = s > 1.0e-8
    d[m] += p[0] / C_TF / _power_int(1 + p[1] * 4 * s[m], 2) / s[m]
    return F, d


def _thak(s, p):
    bs = CBRT_TWO * s
    bs2 = bs * bs
    F = 1.0 + p[0] * bs2 / (1.0 + p[1] * bs * np.arcsinh(bs)) - p[2] * bs / (1.0 + 2 ** (5.0 / 3.0) * bs)
    Fb = (1.0 + p[1] * bs * np.arcsinh(bs)) ** 2
    d = (-(p[0] * p[1] * bs2) / np.sqrt(1 + bs2) + (p[0] * p[1] * bs * np.arcsinh(bs)) + 2.0 * p[0]) / Fb
    m = s > 1.0e-8
    d[m] -= p[2] / (1.0 + 2 ** (5.0 / 3.0) * bs[m]) ** 2 / bs[m]
    return F, d * (CBRT_TWO * CBRT_TWO)


def _b86a(s, p):
    bs = CBRT_TWO * s
    bs2 = bs * bs
    Fb = 1.0 + p[1] * bs2
    return 1.0 + p[0] * bs2 / Fb, 2 * p[0] / (Fb * Fb) * (CBRT_TWO * CBRT_TWO)


def _b86b(s, p):
    bs = CBRT_TWO * s
    bs2 = bs * bs
    Fb = _power_int(1.0 + p[1] * bs2, 4, 5)
    d = (2 * p[0] * (p[1] * bs2 + 5.0)) / (5 * (1.0 + p[1] * bs2) * Fb) * (CBRT_TWO * CBRT_TWO)
    return 1.0 + p[0] * bs2 / Fb, d


def _dk87(s, p):
    bs = CBRT_TWO * s
    bs2 = bs * bs
    Fa = p[0] * bs2 * (1 + p[1] * bs)
    Fb = 1.0 + p[2] * bs2
    d = p[0] * (2.0 + 3.0 * p[1] * bs + p[1] * p[2] * bs2 * bs) / (Fb * Fb) * (CBRT_TWO * CBRT_TWO)
    return 1.0 + Fa / Fb, d


@_tkf0
def _pw86(ss, p):
    s2 = ss * ss
    s4 = s2 * s2
    Fa = 1.0 + p[0] * s2 + p[1] * s4 + p[2] * s2 * s4
    return np.power(Fa, 1.0 / 15.0), 2.0 / 15.0 * (p[0] + 2 * p[1] * s2 + 3 * p[2] * s4) / np.power(Fa, 14.0 / 15.0)


@_tkf0
def _pw91o(ss, p):
    s2 = ss * ss
    s4 = s2 * s2
    ex = np.exp(-p[3] * s2)
    Fa = (p[1] - p[2] * ex) * s2 - p[5] * s4
    Fb = 1.0 + p[0] * ss * np.arcsinh(p[4] * ss) + p[5] * s4
    Fa_s2 = (p[1] - p[2] * ex) - p[5] * s2
    d = 2.0 * (p[1] + (p[3] * s2 - 1) * p[2] * ex - 4.0 * p[5] * s2) / Fb - Fa_s2 * ss / (Fb * Fb) * (
        (p[0] * p[4] * ss) / (p[4] ** 2 * s2 + 1) + p[0] * np.arcsinh(p[4] * ss) + 4.0 * p[5] * s2)
    return 1.0 + Fa / Fb, d


@_tkf0
def _pw91(ss, p):
    s2 = ss * ss
    s4 = s2 * s2
    ex = np.exp(-p[3] * s2)
    ash = np.arcsinh(p[4] * ss)
    Fa = 1.0 + p[0] * ss * ash + (p[1] - p[2] * ex) * s2
    Fb = 1.0 + p[0] * ss * ash + p[5] * s4
    sq = np.sqrt(p[4] ** 2 * s2 + 1)
    Fa_s = p[0] * p[4] * ss / sq + p[0] * ash + 2.0 * ss * (p[1] + 2.0 * p[2] * p[3] * s2 * ex - 2.0 * p[2] * ex)
    d = Fa_s / Fb - Fa / (Fb * Fb) * (p[0] * p[4] * ss / sq + (p[0] * ash + 4.0 * p[5] * s2 * ss))
    m = ss > 1.0e-8
    d[m] /= ss[m]
    return Fa / Fb, d


@_tkf0
def _lg94(ss, p):
    s2 = ss * ss
    s4 = s2 * s2
    s6 = s4 * s2
    s8 = s4 * s4
    s10 = s4 * s6
    s12 = s6 * s6
    Fa = 1.0 + p[0] * s2 + p[1] * s4 + p[2] * s6 + p[3] * s8 + p[4] * s10 + p[5] * s12
    Fb = 1.0 + 1e-8 * s2
    F = np.power(Fa / Fb, p[6])
    d = -2 * p[6] * F * (1e-8 * Fa - Fb * (p[0] + 2 * p[1] * s2 + 3 * p[2] * s4 + 4 * p[3] * s6 + 5 * p[4] * s8
                                          + 6 * p[5] * s10)) / (Fa * Fb)
    return F, d


@_tkf0
def _p92(ss, p):
    s2 = ss * ss
    Fa = p[0] + p[1] * s2 + p[2] * s2 * s2
    Fb = p[0] + p[3] * s2
    return Fa / Fb, (2.0 * p[1] + 4.0 * p[2] * s2) / Fb - (2.0 * p[3] * Fa) / (Fb * Fb)


@_tkf0
def _pbe(ss, p):
    s2 = ss * ss
    Fb = 1.0 + p[1] / p[0] * s2
    Fb2 = Fb * Fb
    F = 1.0 + p[1] * s2 / Fb
    d = 2.0 * p[1] / Fb2
    if len(p) > 2:
        s4 = s2 * s2
        Fb3 = Fb2 * Fb
        F = F + p[2] * s4 / Fb2
        d = d + 4 * p[2] * s2 / Fb3
        if len(p) > 3:
            F = F + p[3] * s4 * s2 / Fb3
            d = d + 6 * p[3] * s4 / (Fb3 * Fb)
    return F, d


@_tkf0
def _p82(ss, p):
    s2 = ss * ss
    s6 = s2 * s2 * s2
    Fb = 1 + s6
    return 1.0 + p[0] * s2 / Fb, p[0] * (2.0 / Fb - 6.0 * s6 / (Fb * Fb))


@_tkf0
def _vjks00(ss, p):
    s2 = ss * ss
    s4 = s2 * s2
    Fa = 1.0 + p[0] * s2 - p[2] * s4 * s2
    Fb = 1.0 + p[1] * s2 + p[2] * s4
    return Fa / Fb, (2.0 * p[0] - 6.0 * p[2] * s4) / Fb - (2.0 * p[1] + 4.0 * p[2] * s2) * Fa / (Fb * Fb)


@_tkf0
def _vt84f(ss, p):
    s2 = ss * ss
    s2 = np.where(s2 < 1.0e-8, 1.0e-8, s2)
    s4 = s2 * s2
    e1, e2 = np.exp(-p[1] * s2), np.exp(-p[1] * s4)
    F = 1.0 + 5.0 / 3.0 * s2 + p[0] * s2 * e1 / (1 + p[0] * s2) + (1 - e2) * (1.0 / s2 - 1.0)
    d = (10.0 / 3.0 + 2.0 * p[0] * e1 * (1.0 - p[1] * s2) / (1 + p[0] * s2)
         - 2.0 * p[0] * s2 * e1 / _power_int(1 + p[0] * s2, 2) + 4.0 * p[1] * s2 * (1.0 / s2 - 1.0) * e2
         - 2.0 * (1 - e2) / s4)
    return F, d


@_tkf0
def _tfvw(ss, p):
    return p[0] + 5.0 / 3.0 * p[1] * ss * ss, 10.0 / 3.0 * p[1] * np.ones_like(ss)


@_tkf0
def _stv(ss, p):
    s2 = ss * ss
    Fb = p[3] + p[2] * s2
    return p[0] + 5.0 / 3.0 * p[1] * s2 / Fb, 5.0 / 3.0 * p[1] * (2.0 / Fb - 2.0 * s2 * p[2] / (Fb * Fb))


@_tkf0
def _pbe2m(ss, p):
    s2 = ss * ss
    Fb = p[0] + p[1] * s2
    return 1.0 + p[2] * s2 / Fb, 2.0 * p[2] / (Fb * Fb)


@_tkf0
def _pg(ss, p):
    s2 = ss * ss
    Fa = np.exp(-p[0] * s2)
    return Fa + 5.0 / 3.0 * p[1] * s2, -2.0 * p[0] * Fa + 10.0 / 3.0 * p[1]


@_tkf0
def _lkt(ss, p):
    s2 = ss * ss
    F = np.empty_like(ss)
    d = np.empty_like(ss)
    m1 = ss > 100.0
    m2 = ss < 1e-5
    m = ~(m1 | m2)
    F[m] = 1.0 / np.cosh(p[0] * ss[m]) + 5.0 / 3.0 * s2[m] * p[1]
    F[m1] = 5.0 / 3.0 * s2[m1] * p[1]
    F[m2] = 1.0 + (5.0 / 3.0 * p[1] - 0.5 * p[0] ** 2) * s2[m2] + 5.0 / 24.0 * p[0] ** 4 * s2[m2] ** 2
    d[m] = 10.0 / 3.0 * p[1] - p[0] * np.sinh(p[0] * ss[m]) / np.cosh(p[0] * ss[m]) ** 2 / ss[m]
    d[m1] = 10.0 / 3.0 * p[1]
    d[m2] = 10.0 / 3.0 * p[1] - p[0] ** 2 + 5.0 / 6.0 * p[0] ** 4 * s2[m2] - 61.0 / 120.0 * p[0] ** 6 * s2[m2] ** 2
    return F, d


# GGA_KEDF_list (gga.py:587-643): name -> (formula, default params)
GGA_FUNCTIONALS = {
    "LKT-VW": (_lkt_mvw, [1.3]), "LKT": (_lkt, [1.3, 1.0]),
    "DK": (_dk, [0.95, 14.28111, -19.5762, -0.05, 9.99802, 2.96085]),
    "LLP": (_llp, [0.0044188, 0.0253]), "LLP91": (_llp, [0.0044188, 0.0253]),
    "OL1": (_ol, [0.00677, 0.0]), "OL": (_ol, [0.00677, 0.0]), "OL2": (_ol, [0.0887, 1.0]),
    "T92": (_thak, [0.0055, 0.0253, 0.072]), "THAK": (_thak, [0.0055, 0.0253, 0.072]),
    "B86A": (_b86a, [0.0039, 0.004]), "B86": (_b86a, [0.0039, 0.004]), "B86B": (_b86b, [0.00403, 0.007]),
    "DK87": (_dk87, [7.0 / 324.0 / (18.0 * np.pi ** 4) ** (1.0 / 3.0), 0.861504, 0.044286]),
    "PW86": (_pw86, [1.296, 14.0, 0.2]),
    "PW91O": (_pw91o, [0.093907, 0.26608, 0.0809615, 100.0, 76.320, 0.57767e-4]),
    "PW91": (_pw91, [0.19645, 0.2747, 0.1508, 100.0, 7.7956, 0.004]),
    "LG94": (_lg94, [(1e-8 + 0.1234) / 0.024974, 29.790, 22.417, 12.119, 1570.1, 55.944, 0.024974]),
    "E00": (_p92, [135.0, 28.0, 5.0, 3.0]), "P92": (_p92, [1.0, 88.3960, 16.3683, 88.2108]),
    "PBE2": (_pbe, [2.0309 / 0.2942, 2.0309]), "PBE3": (_pbe, [-3.7425 / 4.1355, -3.7425, 50.258]),
    "PBE4": (_pbe, [-7.2333 / 1.7107, -7.2333, 61.645, -93.683]), "P82": (_p82, [5.0 / 27.0]),
    "TW02": (_pbe, [0.8438, 0.2319]), "APBE": (_pbe, [0.804, 0.23889]), "APBEK": (_pbe, [0.804, 0.23889]),
    "REVAPBEK": (_pbe, [1.245, 0.23889]), "REVAPBE": (_pbe, [1.245, 0.23889]), "RPBE": (_pbe, [1.9632, 0.01979]),
    "VJKS00": (_vjks00, [0.8944, 0.6511, 0.0431]),
    "LC94": (_pw91, [0.093907, 0.26608, 0.0809615, 100.0, 76.32, 0.000057767]),
    "VT84F": (_vt84f, [2.777028126, 2.777028126 - 40.0 / 27.0]),
    "TF": (_tfvw, [1.0, 0.0]), "VW": (_tfvw, [0.0, 1.0]), "X_TF_Y_VW": (_tfvw, [1.0, 1.0]),
    "TFVW": (_tfvw, [1.0, 1.0]), "STV": (_stv, [1.0, 1.0, 0.01, 1.0]), "PBE2M": (_pbe2m, [1.0, 0.2942, 2.0309]),
    "PG": (_pg, [0.75, 1.0]),
}


def _gradient(rho, grid, sigma=None):
    """DirectField.standard_gradient (field.py:267-281): irfftn(i g rho(G)); with
    sigma the 'supersmooth' gradient (field.py:229-262), times exp(-G^2 sigma^2/2)."""
    rhoG = fft(rho, grid)
    if sigma is None:
        return [ifft(1j * grid.g[i] * rhoG, grid) for i in range(3)]
    return [ifft(grid.g[i] * (rhoG * 1j) * np.exp(-grid.gg * sigma ** 2 / 2.0), grid) for i in range(3)]


def _mgga_ge2(ss, q, p):
    """GE2 (gga.py:492-503), in ss = s / TKF0."""
    s2 = ss * ss
    return p[0] + p[1] * s2 + p[2] * q, 2.0 * p[1], p[2] + 0.0 * q


def _mgga_ge4(ss, q, p):
    """GE4 (gga.py:505-517)."""
    F, d, dq = _mgga_ge2(ss, q, p[:3])
    s2 = ss * ss
    return (F + (p[3] * q * q + p[4] * q * s2 + p[5] * s2 * s2), d + (2.0 * p[4] * q + 4.0 * p[5] * s2),
            dq + (2.0 * p[3] * q + p[4] * s2))


def _mgga_pgsl(ss, q, p):
    """PGSL (gga.py:519-531)."""
    s2 = ss * ss
    Fa = np.exp(-p[1] * s2)
    return Fa + q ** 2 * p[0] + 5.0 / 3.0 * p[2] * s2, -2.0 * p[1] * Fa + 10.0 / 3.0 * p[2], 2.0 * p[0] * q


def _mgga_pgslr(ss, q, p):
    """PGSLr (gga.py:533-545)."""
    F, d, dq = _mgga_pgsl(ss, q, p[2:])
    s2 = ss * ss
    return (F + (-p[0] * q * s2 + p[1] * s2 * s2), d + (-2.0 * p[0] * q + 4.0 * p[1] * s2), dq + (-p[0] * s2))


# MGGA_KEDF_list (gga.py:645-650)
MGGA_FUNCTIONALS = {
    "GE2": (_mgga_ge2, [1.0, 5.0 / 27.0, 20.0 / 9.0]),
    "GE4": (_mgga_ge4, [1.0, 5.0 / 27.0, 20.0 / 9.0, 8.0 / 81.0, -1.0 / 9.0, 8.0 / 243.0]),
    "PGSL": (_mgga_pgsl, [0.25, 40.0 / 27.0, 1.0]),
    "PGSLR": (_mgga_pgslr, [0.40, 0.20, 0.25, 40.0 / 27.0, 1.0]),
}


def _laplacian(f, grid, sigma=None):
    """DirectField.laplacian(force_real=True) (field.py:379-386)."""
    F = fft(f, grid)
    if sigma is None or sigma == 0:
        return ifft(-grid.gg * F, grid)
    return ifft(-grid.gg * F * np.exp(-grid.gg * sigma ** 2 / 2.0), grid)


def gga(rho, grid, functional="LKT", params=None, calc=("E", "V"), gga_remove_vw=None, sigma=None, mgga=False):
    """GGA (kedf/gga.py:1212-1325); sigma smooths the density gradient (:1246-1250);
    mgga: the Laplacian-level functionals of MGGA_KEDF_list (:1226-1230, 1254-1257,
    1305-1308), without stress."""
    name = functional.upper()
    fn, p0 = (MGGA_FUNCTIONALS if mgga else GGA_FUNCTIONALS)[name]
    p = list(p0)
    if params is not None:
        params = [params] if isinstance(params, (int, float)) else list(params)
        p[:min(len(params), len(p))] = params[:len(p)]
    rhom = rho.copy()
    rhom[rhom < 1e-16] = 1e-16
    rho23 = _power_int(rhom, 2, 3)
    rho53 = rho23 * rhom
    tf = C_TF * rho53
    rho43 = rho23 * rho23
    rho83 = rho43 * rho43
    grad = _gradient(rho, grid, sigma)
    s = np.sqrt(_power_int(grad[0], 2) + _power_int(grad[1], 2) + _power_int(grad[2], 2)) / rho43
    s[s < 1e-16] = 1e-16
    if mgga:
        q = _laplacian(rho, grid, sigma) / (TKF0 ** 2) / rho53
        F, dFds2, dFdq = fn(s / TKF0, q, p)
        dFds2 = dFds2 / (TKF0 * TKF0)
    else:
        F, dFds2 = fn(s, p)
    if gga_remove_vw is not None:
        pa = float(gga_remove_vw) if isinstance(gga_remove_vw, (int, float)) else 1.0
        Fv, dv = _tfvw(s, [0.0, pa])
        F, dFds2 = F - Fv, dFds2 - dv
    out = {"E": (tf * F).sum() * grid.dV}
    if "V" in calc or "S" in calc:
        pot1 = 5.0 / 3.0 * C_TF * rho23 * F - 4.0 / 3.0 * tf * dFds2 * s * s / rhom
        p3 = [fft(tf * dFds2 * grad[i] / rho83, grid) for i in range(3)]
        pot3G = grid.g[0] * p3[0] + grid.g[1] * p3[1] + grid.g[2] * p3[2]
        out["V"] = pot1 - ifft(1j * pot3G, grid)
        if mgga:
            out["V"] = out["V"] + tf * dFdq * (-5.0 / 3.0 * q / rhom)
            out["V"] = out["V"] + _laplacian(tf * dFdq * (1.0 / (TKF0 ** 2) / rho53), grid, sigma)
    if "S" in calc:
        if mgga:
            raise AttributeError("Stress not support MGGA yet")
        vkin2 = tf * dFds2 / rho83
        P = out["E"] - (pot1 * rho).sum() * grid.dV
        for i in range(3):
            P -= (grad[i] * grad[i] * vkin2).sum() * grid.dV
        S = np.zeros((3, 3))
        for i in range(3):
            S[i, i] = P
            for j in range(i, 3):
                S[i, j] -= (vkin2 * grad[i] * grad[j]).sum() * grid.dV
                S[j, i] = S[i, j]
        out["S"] = S / grid.volume
    return out


# --------------------------------------------------------------------------
# stress (calcType 'S'): 3x3 tensors in Ha/Bohr^3
# --------------------------------------------------------------------------
_SYM6 = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]


def tf_stress(grid, energy):
    """ThomasFermiStress (kedf/tf.py:52-63): -2/3 E/V on the diagonal."""
    return np.eye(3) * (-2.0 / 3.0 * energy / grid.volume)


def vw_stress(rho, grid, y=1.0):
    """vonWeizsackerStress (kedf/vw.py:97-111): -(y/4) dV/V sum d_i rho d_j rho / rho,
    the gradients by irfftn of i g_i rho(G)."""
    g = grid.g
    rhoG = fft(rho, grid)
    d = [ifft(1j * g[i] * rhoG, grid) for i in range(3)]
    s = np.zeros((3, 3))
    for i, j in _SYM6:
        s[i, j] = s[j, i] = (-0.25 / grid.volume * grid.dV * np.einsum("ijk->", d[i] * d[j] / rho)).real * y
    return s


def lindhard_derivative(eta, mu):
    """LindhardDerivative (kedf/kernel.py:197-211), returned times eta."""
    eta = np.asarray(eta, dtype=np.float64)
    out = np.zeros_like(eta)
    atol = 1.0e-10
    c0 = (eta > atol) & (np.abs(eta - 1.0) > atol)
    c1 = eta < atol
    c2 = np.abs(eta - 1.0) < atol
    e = eta[c0]
    A = np.log(np.abs((1.0 + e) / (1.0 - e)))
    out[c0] = (0.5 / e - 0.25 * (e ** 2 + 1.0) / e ** 2 * A) / (0.5 + 0.25 * (1 - e ** 2) / e * A) ** 2 + 6.0 * e * mu
    out[c1] = -2.0 * eta[c1] * (1.0 / 3.0 - 3.0 * mu)
    out[c2] = -48
    return out * eta


def wt_stress(rho, grid, energy, y=1.0, alpha=5.0 / 6.0, beta=5.0 / 6.0):
    """WTStress (kedf/wt.py:75-106) with rho0 = the mean density."""
    rho0 = rho.sum() / grid.nnr
    g, invgg, q, mask = grid.g, grid.invgg, grid.q, grid.mask
    tkf = float(2.0 * (3.0 * rho0 * np.pi ** 2) ** (1.0 / 3.0))
    rA = fft(rho ** alpha, grid) / grid.volume
    rB = np.conjugate(fft(rho ** beta, grid)) / grid.volume
    DD = lindhard_derivative(q / tkf, y) * rA * rB
    s = np.zeros((3, 3))
    for i, j in _SYM6:
        fac = 1.0 / 3.0 if i == j else 0.0
        den = (g[i][mask] * g[j][mask] * invgg[mask] - fac) * DD[mask]
        s[i, j] = s[j, i] = np.einsum("i->", den).real
    s *= np.pi ** 2 / (alpha * beta * rho0 ** (alpha + beta - 2) * tkf / 2.0)
    for i in range(3):
        s[i, i] -= 2.0 / 3.0 * energy / grid.volume
    return s


def lda_stress(rho, grid, energy, potential):
    """_LDAStress (xc/semilocal_xc.py:343-346): (E - int v rho) / V on the diagonal."""
    P = energy - np.sum(potential * rho) * grid.dV
    return np.eye(3) * P / grid.volume


def hartree_stress(rho, grid, energy):
    """HartreeFunctionalStress (hartree.py:67-90)."""
    g, invgg, mask = grid.g, grid.invgg, grid.mask
    rhoG = fft(rho, grid)
    rhoG2 = rhoG * np.conjugate(rhoG) * invgg * invgg
    s = np.zeros((3, 3))
    for i, j in _SYM6:
        e = np.sum((g[i][mask] * g[j][mask]) * rhoG2[mask])
        s[i, j] = s[j, i] = e.real * 8.0 * np.pi / grid.volume ** 2
        if i == j:
            s[i, j] -= energy / grid.volume
    return s


def vline_deriv(grid, gp, vp):
    """_PP_Derivative_One (pseudo/__init__.py:454-460): splev(q, tck, der=1) of the
    spline of ReadPseudo.get_vloc_interp (:689-706) below max(gp), 0 above."""
    tck = splrep(gp[1:], vp[1:], k=3)
    q = grid.q
    out = np.zeros_like(q)
    m = q < np.max(gp)
    out[m] = splev(q[m], tck, der=1)
    return out


def _invq(grid):
    q = grid.q.copy()  # grid.py:544-553: G = 0 -> 0
    q[0, 0, 0] = 1.0
    inv = 1.0 / q
    inv[0, 0, 0] = 0.0
    return inv


def pp_stress(pp, rho, energy=None):
    """LocalPseudo.stress (pseudo/__init__.py:248-258): _StressPME (:573-611) or
    _Stress (:479-503).  ``pp`` is an oracle LocalPseudo."""
    g = pp.grid
    if energy is None:
        energy = pp(rho, calc=("E",))["E"]
    rhoG = fft(rho, g)
    gv, mask, invq = g.g, g.mask, _invq(g)
    s = np.zeros((3, 3))
    if pp.PME:
        rhoGB = np.conjugate(rhoG) * bspline_barray(g, pp.order)
        frac = scaled_positions(pp.pos, g.lattice)
        for sp_i, (gp, vp) in enumerate(pp.tables):
            sel = pp.species == sp_i
            if not sel.any():
                continue
            Q = pme_qarray(g, frac[sel], np.ones(sel.sum()), pp.order)
            rhoGBV = rhoGB * vline_deriv(g, gp, vp) * fft(Q, g)
            for i, j in _SYM6:
                den = (gv[i][mask] * gv[j][mask]) * rhoGBV[mask] * invq[mask]
                s[i, j] -= np.einsum("i->", den).real / g.volume ** 2
        s *= 2.0 * g.nnr
        for i in range(3):
            for j in range(i, 3):
                s[j, i] = s[i, j]
            s[i, i] -= energy
        return s / g.volume
    v = np.zeros(tuple(g.nrG), dtype=np.complex128)
    for sp_i, (gp, vp) in enumerate(pp.tables):
        dv = vline_deriv(g, gp, vp)
        for a in np.nonzero(pp.species == sp_i)[0]:
            v += dv * np.exp(1j * np.einsum("lijk,l->ijk", gv, pp.pos[a]))
    rGV = rhoG * v * invq
    for i, j in _SYM6:
        den = (gv[i][mask] * gv[j][mask]) * rGV[mask]
        s[i, j] = s[j, i] = -np.einsum("i->", den).real / g.volume * 2.0
        if i == j:
            s[i, j] -= energy
    return s / g.volume


def _ewald_sfactor(grid, eta):
    """The six sfactor planes of Stress_rec / Stress_rec_PME (ewald.py:738-745, :941-947)."""
    gv, gg, invgg = grid.g, grid.gg, grid.invgg
    out = []
    for i, j in _SYM6:
        f = gv[i] * gv[j] * 2.0 * invgg * (1 + gg / (4.0 * eta))
        if i == j:
            f = f - 1.0
        out.append(f)
    return out


def ewald_stress(ew):
    """ewald.stress (ewald.py:523-538): Stress_real (:609-662) + Stress_rec_PME
    (:915-968) or Stress_rec (:719-763).  ``ew`` is an oracle Ewald."""
    g = ew.grid
    R, Rcut = ew._images()
    es = np.sqrt(ew.eta)
    S6 = np.zeros(6)
    for ia in range(len(ew.pos)):
        rj = (ew.pos[None, :, :] - R[:, None, :]).reshape(-1, 3)
        qj = np.broadcast_to(ew.q[None, :], (len(R), len(ew.q))).ravel()
        Rij = ew.pos[ia][None, :] - rj
        d = np.sqrt((Rij * Rij).sum(-1))
        m = (d < Rcut) & (d > 0.001)
        Rij, d, qj = Rij[m], d[m], qj[m]
        Rv = np.stack([Rij[:, i] * Rij[:, j] / d ** 2 for i, j in _SYM6], axis=1)
        S6 += ew.q[ia] * np.einsum("i,ij->j", qj * (2 * es / np.sqrt(np.pi) * np.exp(-ew.eta * d ** 2)
                                                    + sp.erfc(es * d) / d), Rv)
    S6 *= -0.5 / g.volume
    mask, gg, invgg = g.mask, g.gg, g.invgg
    if ew.PME:
        Q, _ = ew._qgrid()
        strf = fft(Q, g) * bspline_barray(g, ew.order)
        scale = 2.0 * 2.0 * np.pi / g.volume ** 2 / g.dV ** 2
    else:
        strf = np.zeros(tuple(g.nrG), dtype=np.complex128)
        for a in range(len(ew.pos)):
            strf += np.exp(-1j * np.einsum("lijk,l->ijk", g.g, ew.pos[a])) * ew.q[a]
        scale = 4.0 * np.pi / g.volume ** 2
    w = (np.conjugate(strf) * strf)[mask] * np.exp(-gg[mask] / (4.0 * ew.eta)) * invgg[mask]
    rec6 = np.array([np.einsum("i,i->", w, f[mask]).real for f in _ewald_sfactor(g, ew.eta)]) * scale
    sg0 = np.sum(ew.q) ** 2 * 4.0 * np.pi * (1.0 / (4.0 * ew.eta * g.volume ** 2) / 2.0)
    s = np.zeros((3, 3))
    for k, (i, j) in enumerate(_SYM6):
        s[i, j] = s[j, i] = S6[k] + rec6[k] + (sg0 if i == j else 0.0)
    return s


# --------------------------------------------------------------------------
# total functional
# --------------------------------------------------------------------------
class Total:
    """TotalFunctional.get_energy_potential (total_functional.py:115-146): sum of terms
    plus the Ewald energy.  ``terms`` are callables (rho, calc) -> {'E','V'}."""

    def __init__(self, grid, terms, ewald_energy=None):
        self.grid, self.terms, self.ewald_energy = grid, terms, ewald_energy

    def __call__(self, rho, calc=("E", "V")):
        E = 0.0
        V = np.zeros_like(rho) if "V" in calc else None
        parts = {}
        for name, fn in self.terms:
            o = fn(rho, calc)
            if "E" in calc:
                parts[name] = o["E"]
                E += o["E"]
            if "V" in calc:
                V += o["V"]
        if self.ewald_energy is not None and "E" in calc:
            parts["II"] = self.ewald_energy
            E += self.ewald_energy
        return {"E": E, "V": V, "parts": parts}


def make_terms(grid, kedf="TFVW", xc=True, hartree=True, pseudo=None, **kw):
    """KEDF name dispatch (kedf/__init__.py:27-69) for TF, VW, TFVW, WT, LWT."""
    terms = []
    names = {"TF": ("TF",), "VW": ("VW",), "TFVW": ("TF", "VW"), "WT": ("TF", "VW", "WT-NL"),
             "LWT": ("TF", "VW", "LWT-NL")}[kedf.upper()]
    for n in names:
        if n == "TF":
            terms.append(("TF", lambda r, c: tf(r, grid, kw.get("x", 1.0), c)))
        elif n == "VW":
            terms.append(("VW", lambda r, c: vw(r, grid, kw.get("y", 1.0), c)))
        elif n == "WT-NL":
            wt = WT(x=kw.get("x", 1.0), alpha=kw.get("alpha", 5.0 / 6.0), beta=kw.get("beta", 5.0 / 6.0),
                    rho0=kw.get("rho0"))
            terms.append(("NL", lambda r, c, wt=wt: wt(r, grid, c)))
        elif n == "LWT-NL":
            lw = LWT(**{k: v for k, v in kw.items() if k in (
                "x", "alpha", "beta", "etamax", "neta", "interp", "kdd", "ratio", "nsp", "delta", "kfmin", "kfmax", "ldw")})
            terms.append(("NL", lambda r, c, lw=lw: lw(r, grid, c)))
    if xc:
        terms.append(("XC", lambda r, c: lda(r, grid, c)))
    if hartree:
        terms.append(("H", lambda r, c: _hartree_fn(r, grid, c)))
    if pseudo is not None:
        terms.append(("PP", lambda r, c: pseudo(r, c)))
    return terms


# --------------------------------------------------------------------------
# density optimisation
# --------------------------------------------------------------------------
def optimize(evaluator, rho0, grid, method="TN", maxiter=100, maxfun=50, maxls=30, econv=1e-5,
             c1=1e-4, c2=0.2, xtol=1e-12, ncheck=2, maxcor=6, h0=1.0, trace=None):
    """Optimization.optimize_rho (optimization/optimization.py:283-525) for one spin,
    algorithm EMM, vector 'Orthogonalization', line search = scipy line_search_wolfe1
    started at theta=1 (math_utils.py:37-52: alpha0 is not forwarded); DIIS runs the
    reference's damped fixed point instead (no line search, _diis_iteration).
    ``evaluator(rho, calc)`` returns {'E','V'}.  Returns (rho, info)."""
    from scipy.optimize._linesearch import line_search_wolfe1
    dV = grid.dV
    mask = rho0 > 0
    phi = np.where(mask, np.sqrt(np.where(mask, rho0, 0.0)), 1e-300)
    phi *= np.sqrt(rho0.sum() / (phi * phi).sum())
    rho = phi * phi
    f = evaluator(rho, ("E", "V"))
    N = rho.sum() * dV
    mu = (f["V"] * rho).sum() * dV / N
    res = (f["V"] - mu) * phi
    resA, dirA = [res], []
    Ehist = [f["E"]]
    lb = {"s": [], "y": [], "rho": []}
    converged = 2
    nfev = 1
    for it in range(1, maxiter):
        if method == "DIIS":
            phi, rho, f, N, mu, res = _diis_iteration(evaluator, phi, resA[-1], N, dV)
            nfev += 2
            resA.append(res)
            Ehist.append(f["E"])
            if trace is not None:
                trace.append((it, f["E"], (res * res).sum() * dV))
            if _check_conv(Ehist, econv, ncheck):
                converged = 0
                break
            if len(resA) > 2:
                resA.pop(0)
            continue
        if method == "TN":
            p, nd = _tn_direction(evaluator, resA[-1], phi, mu, maxfun)
            nfev += nd
        elif method == "LBFGS":
            p = _lbfgs_direction(resA, lb, h0)
        else:
            p = _cg_direction(resA, dirA, method)
        p, theta0 = _orth_norm(p, phi, dV)
        if (f["V"] * phi * p).sum() * 2.0 > 0:                   # :373-380 uphill -> steepest descent
            p, theta0 = _orth_norm(-resA[-1], phi, dV)

        cache = {}

        def vd(theta):
            key = float(theta)
            if key not in cache:
                nphi = phi * np.cos(theta) + p * np.sin(theta)
                fr = evaluator(nphi * nphi, ("E", "V"))
                p2 = p * np.cos(theta) - phi * np.sin(theta)
                grad = 2.0 * (fr["V"] * nphi * p2).sum() * dV
                cache.clear()
                cache[key] = (fr["E"], grad, nphi, fr)
            return cache[key]

        v0 = (f["E"], 2.0 * (f["V"] * phi * p).sum() * dV, phi, f)
        cache[0.0] = v0
        cnt = [0]

        def fn(x):
            cnt[0] += 1
            return vd(x)[0]

        def fp(x):
            return vd(x)[1]

        ls = line_search_wolfe1(fn, fp, 0.0, 1.0, gfk=v0[1], old_fval=v0[0], c1=c1, c2=c2,
                                amax=np.pi, amin=0.0, xtol=xtol)
        nfev += cnt[0]
        theta = ls[0]
        if theta is None:
            converged = 1
            break
        _, _, nphi, fnew = vd(theta)
        old_phi, phi = phi, nphi
        rho = phi * phi
        f = fnew
        N = rho.sum() * dV
        mu = (f["V"] * rho).sum() * dV / N
        res = (f["V"] - mu) * phi
        resA.append(res)
        if method == "LBFGS":
            _lbfgs_update(lb, phi - old_phi, resA[-1] - resA[-2], maxcor)
        Ehist.append(f["E"])
        resN = (res * res).sum() * dV
        if trace is not None:
            trace.append((it, f["E"], resN))
        if _check_conv(Ehist, econv, ncheck):
            converged = 0
            break
        dirA.append(p)
        if len(resA) > 2:
            resA.pop(0)
        if len(dirA) > 2:
            dirA.pop(0)
    return rho, {"converged": converged, "mu": mu, "energy": f["E"], "niter": it, "nfev": nfev,
                 "dP": float((res * res).sum() * dV)}


def _check_conv(E, econv, ncheck):
    """check_converge (optimization.py:527-540)."""
    if len(E) - 1 < ncheck:
        return False
    for i in range(ncheck):
        if abs(E[-2 - i] - E[-1]) > econv:
            return False
    return True


def _orth_norm(p, phi, dV):
    """OrthogonalNormalization (optimization.py:205-226)."""
    Ne = (phi * phi).sum() * dV
    p = p - ((p * phi).sum() * dV / Ne) * phi
    pN = (p * p).sum() * dV
    theta = np.sqrt(pN / Ne)
    return p * np.sqrt(Ne / pN), theta


def _tn_direction(evaluator, res0, phi, mu, maxfun):
    """get_direction_TN (optimization.py:92-148): CG on finite-difference Hessian products."""
    eps = 1.0e-9
    d = np.zeros_like(res0)
    r = -res0.copy()
    p = r.copy()
    r0 = (r * r).sum()
    rconv = r0 * 0.1
    best = d
    rl = [1e10]
    it = 0
    for it in range(maxfun):
        phi1 = phi + eps * p
        fv = evaluator(phi1 * phi1, ("V",))
        Ap = ((fv["V"] - mu) * phi1 - res0) / eps
        pAp = (p * Ap).sum()
        if pAp < 0.0:
            if it == 0:
                d = r0 / pAp * p
            break
        a = r0 / pAp
        d = d + a * p
        r = r - a * Ap
        r1 = (r * r).sum()
        if r1 < min(rl):
            best = d.copy()
        rl.append(r1)
        if r1 < rconv:
            break
        elif r1 > 1000 * min(rl[:-1]):
            d = best
            break
        elif it > 10 and abs(r0 - r1) < 0.1 * r0:
            d = best
            break
        beta = r1 / r0
        r0 = r1
        p = r + beta * p
    return d, it + 1


def _lbfgs_update(lb, dx, dg, bound):
    """LBFGS.update (math_utils.py:307-325): keeps at most bound+1 pairs."""
    if len(lb["s"]) > bound:
        lb["s"].pop(0)
        lb["y"].pop(0)
        lb["rho"].pop(0)
    lb["s"].append(dx)
    lb["y"].append(dg)
    lb["rho"].append(1.0 / (dg * dx).sum())


def _lbfgs_direction(resA, lb, h0):
    """Optimization.get_direction_LBFGS (optimization.py:150-171); first loop skips i=0."""
    q = -resA[-1]
    al = np.zeros(len(lb["s"]))
    for i in range(len(lb["s"]) - 1, 0, -1):
        a = lb["rho"][i] * (lb["s"][i] * q).sum()
        al[i] = a
        q = q - a * lb["y"][i]
    if not h0:
        gamma = 1.0 if len(lb["s"]) < 1 else (lb["s"][-1] * lb["y"][-1]).sum() / (lb["y"][-1] * lb["y"][-1]).sum()
        d = gamma * q
    else:
        d = h0 * q
    for i in range(len(lb["s"])):
        b = lb["rho"][i] * (lb["y"][i] * d).sum()
        d = d + lb["s"][i] * (al[i] - b)
    return d


def _cg_direction(resA, dirA, method="CG-HS"):
    """get_direction_CG (math_utils.py:326-349) and get_direction_GD (:352-354).
    CG-CD's beta is a field, -(r*r)/sum(d r_prev), as in the reference; any other
    CG name falls to the last branch (Fletcher-Reeves)."""
    if method == "GD":
        return -resA[-1]
    if len(resA) == 1:
        beta = 0.0
    elif method in ("CG-HS", "CG") and len(dirA) > 0:
        dr = resA[-1] - resA[-2]
        beta = (resA[-1] * dr).sum() / (dirA[-1] * dr).sum()
    elif method == "CG-PR":
        beta = max((resA[-1] * (resA[-1] - resA[-2])).sum() / (resA[-2] ** 2).sum(), 0.0)
    elif method == "CG-DY" and len(dirA) > 0:
        beta = (resA[-1] ** 2).sum() / (dirA[-1] * (resA[-1] - resA[-2])).sum()
    elif method == "CG-CD" and len(dirA) > 0:
        beta = -(resA[-1] ** 2) / (dirA[-1] * resA[-2]).sum()
    elif method == "CG-LS" and len(dirA) > 0:
        beta = (resA[-1] * (resA[-1] - resA[-2])).sum() / (dirA[-1] * resA[-2]).sum()
    else:
        beta = (resA[-1] ** 2).sum() / (resA[-2] ** 2).sum()
    if not dirA:
        return -resA[-1]
    return -resA[-1] + beta * dirA[-1]


def _diis_iteration(evaluator, phi, res, Ncur, dV):
    """One iteration of the reference's DIIS (optimization.py:327-333, :429-441,
    :471-485): p = -r left unscaled ('Scaling'); phi + 0.1 p renormalised to the
    current electron count and evaluated for V only; then phi + 0.1 p from the new
    residual, whose factor rho.N / rho.integral() is 1 (both the integral of the
    same fresh field), evaluated for E and V.  Returns (phi, rho, f, N, mu, res)."""
    nphi = phi + 0.1 * (-res)
    nrho = nphi * nphi
    norm = Ncur / (nrho.sum() * dV)
    nrho = nrho * norm
    nphi = nphi * np.sqrt(norm)
    fv = evaluator(nrho, ("V",))
    phi = nphi
    rho = phi * phi
    N = rho.sum() * dV
    mu = (fv["V"] * rho).sum() * dV / N
    res = (fv["V"] - mu) * phi
    phi = phi + 0.1 * (-res)
    rho = phi * phi
    f = evaluator(rho, ("E", "V"))
    N = rho.sum() * dV
    mu = (f["V"] * rho).sum() * dV / N
    res = (f["V"] - mu) * phi
    return phi, rho, f, N, mu, res


# --------------------------------------------------------------------------
# density mixing and OE-SCF
# --------------------------------------------------------------------------
def pred_matrix(grid, predtype, predcoef):
    """SpecialPrecondition.matrix (mixer/mixer.py:28-40): None -> 1, kerker
    (:72-80), inverse_kerker (:82-95, 0 at G = 0), resta (:97-113, 1 at G = 0)."""
    pc = list(predcoef) + [1.0] * (3 - len(predcoef)) if predcoef else [0.8, 1.0, 1.0]
    gg = grid.gg
    if predtype is None:
        return np.ones(gg.shape)
    if predtype == "kerker":
        return pc[0] * np.minimum(gg / (gg + pc[1] ** 2), pc[2])
    if predtype == "inverse_kerker":
        g = gg.copy()
        g[0, 0, 0] = 1.0
        m = pc[0] ** 2 / g + 1.0
        m[0, 0, 0] = 0.0
        return m
    if predtype == "resta":
        q = np.sqrt(gg)
        q[0, 0, 0] = 1.0
        m = (pc[1] ** 2 * np.sin(q * pc[2]) / (pc[0] * q * pc[2]) + gg) / (pc[1] ** 2 + gg)
        m[0, 0, 0] = 1.0
        return m
    raise ValueError(predtype)


def pred_mask(grid, predecut):
    """SpecialPrecondition.mask (mixer.py:56-70): |G|^2 above gmax."""
    gg = grid.gg
    if predecut is None:
        return np.zeros(gg.shape, dtype=bool)
    if predecut < 2:
        gmax = max(gg[:, 0, 0].max(), gg[0, :, 0].max(), gg[0, 0, :].max()) + 2
    else:
        gmax = 2.0 * predecut
    return gg > gmax


def precondition(nin, nout, grid, predtype, predcoef, predecut, drho=None, residual=None, coef=0.7):
    """SpecialPrecondition.compute (mixer.py:126-140)."""
    nin_g = fft(nin, grid)
    results = nin_g.copy()
    if drho is not None:
        results += fft(drho, grid)
    if residual is not None:
        results += fft(residual, grid) * pred_matrix(grid, predtype, predcoef)
    mask = pred_mask(grid, predecut)
    if mask.any():
        results[mask] = nin_g[mask] * (1 - coef) + coef * fft(nout, grid)[mask]
    return ifft(results, grid)


class PulayMixer:
    """PulayMixer (mixer/pulay.py:8-120), Kresse and Furthmueller (1996)."""

    def __init__(self, grid, predtype=None, predcoef=(0.8, 1.0, 1.0), maxm=5, coef=0.7, delay=0, predecut=None,
                 restarted=False):
        self.grid, self.predtype, self.predcoef, self.predecut = grid, predtype, list(predcoef), predecut
        self.maxm, self.coef, self.delay, self.restarted = maxm, coef, delay, restarted
        self.it = 0
        self.dr_mat = self.dn_mat = None
        self.prev_density = self.prev_residual = None

    def _pred(self, nin, nout, drho=None, residual=None, coef=0.7):
        return precondition(nin, nout, self.grid, self.predtype, self.predcoef, self.predecut, drho, residual, coef)

    def __call__(self, nin, nout, coef=None):
        from scipy import linalg
        coef = self.coef if coef is None else coef
        self.it += 1
        r = nout - nin
        if self.it == 1 and self.delay < 1:
            results = self._pred(nin, nout, residual=r * coef)
        elif self.it > self.delay:
            if self.restarted and (self.it - self.delay) % (self.maxm + 1) == 0:
                self.dr_mat = self.dn_mat = None
            dn = nin - self.prev_density
            dr = r - self.prev_residual
            if self.dr_mat is None:
                self.dr_mat, self.dn_mat = dr[None].copy(), dn[None].copy()
            elif len(self.dr_mat) < self.maxm:
                self.dr_mat = np.concatenate((self.dr_mat, dr[None]))
                self.dn_mat = np.concatenate((self.dn_mat, dn[None]))
            else:
                self.dr_mat = np.roll(self.dr_mat, -1, axis=0)
                self.dr_mat[-1] = dr
                self.dn_mat = np.roll(self.dn_mat, -1, axis=0)
                self.dn_mat[-1] = dn
            ns = len(self.dr_mat)
            amat = np.empty((ns, ns))
            b = np.empty(ns)
            for i in range(ns):
                for j in range(i + 1):
                    amat[i, j] = amat[j, i] = (self.dr_mat[i] * self.dr_mat[j]).sum()
                b[i] = -(self.dr_mat[i] * r).sum()
            try:
                x = linalg.solve(amat, b, assume_a="sym")
                drho = x[0] * self.dn_mat[0]
                res = r + x[0] * self.dr_mat[0]
                for i in range(1, ns):
                    drho += x[i] * self.dn_mat[i]
                    res += x[i] * self.dr_mat[i]
                res *= coef
                results = self._pred(nin, nout, drho, res, coef)
            except Exception:
                results = self._pred(nin, nout, residual=r * coef, coef=coef)
        else:
            results = nout.copy()
        self.prev_density = nin + 0.0
        self.prev_residual = r + 0.0
        return results


class LinearMixer:
    """LinearMixer (mixer/linear.py:4-35)."""

    def __init__(self, grid, predtype="inverse_kerker", predcoef=(0.8, 1.0, 1.0), coef=0.7, delay=0, predecut=None):
        self.grid, self.predtype, self.predcoef, self.predecut = grid, predtype, list(predcoef), predecut
        self.coef, self.delay, self.it = coef, delay, 0

    def __call__(self, nin, nout, coef=None):
        self.it += 1
        coef = self.coef if coef is None else coef
        if self.it > self.delay and coef < 1.0 - 1e-10:
            return precondition(nin, nout, self.grid, self.predtype, self.predcoef, self.predecut,
                                residual=(nout - nin) * coef, coef=coef)
        return nout.copy()


def oescf(terms, emb_terms, rho0, grid, mixer, econv, maxiter=100, method="CG-HS", opt_kw=None, ewald_energy=None):
    """OESCF.run (optimization/scf.py:37-119): ``terms`` the inner functional (vW
    and the rest, plus the Ewald energy), ``emb_terms`` the frozen embedding
    part, both as make_terms lists; the inner optimisation is ``optimize``.
    Returns (rho, {'history', 'iter'})."""
    opts = dict(opt_kw or {})
    ncharges = rho0.sum() * grid.dV
    rho = rho0.copy()
    state = {"econv": econv}
    history, it, dp_norm, dp_prev = [], 0, None, None
    for _ in range(maxiter):
        it += 1
        norm = ncharges * 1e-1 if it == 1 else (ncharges * 1e-3 if it == 2 else dp_norm)
        if it == 1:
            state["econv"] = 1e10
        e = max(norm * 1e-2, 1e-7 * ncharges)
        if e < state["econv"]:
            state["econv"] = e
        rho_prev = rho.copy()
        emb = Total(grid, emb_terms)(rho, ("E", "V"))
        v = emb["V"]
        extenergy = emb["E"] - (v * rho).sum() * grid.dV
        ev = Total(grid, list(terms) + [("EXT", lambda r, c, v=v: {"E": (v * r).sum() * grid.dV, "V": v})],
                   ewald_energy=ewald_energy)
        rho, info = optimize(ev, rho, grid, method=method, econv=state["econv"], **opts)
        energy = info["energy"] + extenergy
        error = abs(energy - history[-1]) if history else abs(energy)
        history.append(energy)
        dp = hartree(rho - rho_prev, grid, ("E",))["E"]
        if it == 1:
            dp_norm = dp_prev = dp
        else:
            dp_norm, dp_prev = dp_prev, dp
            dp_norm = (dp_norm + dp_prev) / 2
        if mixer is not None:
            rho = mixer(rho_prev, rho)
        if error < econv:
            break
    return rho, {"history": history, "iter": it}


# --------------------------------------------------------------------------
# Fourier interpolation between grids of one cell
# --------------------------------------------------------------------------
def grid_map_index(nr, nr2):
    """grid_map_index (utils/utils.py:50-78) for half grids: the coarse half
    spectrum's indices in the fine one, and whether nr2 is the fine grid."""
    coarse, fine = np.array(nr, dtype=int), np.array(nr2, dtype=int)
    lfine = True
    if np.all(fine < coarse) or (not np.all(fine > coarse) and not np.prod(fine) > np.prod(coarse)):
        coarse, fine, lfine = fine, coarse, False
    coarse = np.minimum(fine, coarse)
    dnr = coarse.copy()
    dnr[:2] = coarse[:2] // 2
    index = np.mgrid[:coarse[0], :coarse[1], :coarse[2]].reshape((3, -1))
    for i in range(3):
        m = index[i] > dnr[i]
        index[i][m] += fine[i] - coarse[i]
    return index, lfine


def grid_map(f, grid, nr_dst):
    """grid_map_data(data, nr) (utils/utils.py:80-128): the field on the grid of
    the same cell with nr_dst points."""
    F = fft(f, grid)
    g2 = Grid(grid.lattice, nr_dst)
    nr1, nr2 = F.shape, tuple(g2.nrG)
    G = np.zeros(nr2, dtype=np.complex128)
    index, lfine = grid_map_index(nr1, nr2)
    bd = np.minimum(nr1, nr2)
    if lfine:
        G[index[0], index[1], index[2]] = F[:bd[0], :bd[1], :bd[2]].ravel()
    else:
        G[:bd[0], :bd[1], :bd[2]] = F[index[0], index[1], index[2]].reshape(bd)
    return ifft(G, g2)


# --------------------------------------------------------------------------
# density-independent MGP kernels
# --------------------------------------------------------------------------
def mgp_kernel(grid, rho0, maxpoints=1000, symmetrization=None, lumpfactor=0.2, revke=True):
    """MGPKernel (kedf/kernel.py:251-263) with MGPKernelTable (:267-322) on the 3-D
    grid (splrep of LindhardFunction(eta, 1, 1) on 10000 log-spaced points from
    1e-4 to 52, splev with ext=3) plus MGPOmegaE (:408-440) at Ne = rho0 V."""
    from scipy.interpolate import splev, splrep
    q = np.sqrt(grid.gg)
    tkf = 2.0 * (3.0 * rho0 * np.pi ** 2) ** (1.0 / 3.0)
    eta = q / tkf
    gp = np.logspace(np.log10(1e-4), np.log10(52), num=10000)
    tab = splrep(gp, lindhard(gp, 1.0, 1.0))
    dt = 1.0 / maxpoints
    cTF = 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
    coe = 4.0 / 5.0 * cTF * 5.0 / 6.0 * dt
    k = np.zeros_like(eta)
    for i in range(1, maxpoints + 1):
        t = i * dt
        t16 = t ** (-2.0 / 3.0) if symmetrization == "Geometric" else t ** (1.0 / 6.0)
        k += splev(eta / np.cbrt(t), tab, ext=3) / t16
    if symmetrization == "Arithmetic":
        k = 0.5 * (k * coe + wt_kernel_table(eta))
    elif symmetrization == "Geometric":
        k *= 2.0 * coe
    else:
        k *= coe
    k[0, 0, 0] = 0.0
    if lumpfactor is not None:
        c, b = 1.0, None
        if isinstance(lumpfactor, (list, tuple)):
            a = lumpfactor[0]
            if len(lumpfactor) > 1:
                b = lumpfactor[1]
            if len(lumpfactor) > 2:
                c = lumpfactor[2]
        else:
            a = lumpfactor
        if b is None:
            a = float(a / (rho0 * grid.volume) ** (2.0 / 3.0))
            b = a
        qq = q.copy()
        qq[0, 0, 0] = 1.0
        gg = qq ** 2
        if revke:
            corr = 4 * np.pi * sp.erf(c * gg) ** 2 * a * np.exp(-gg * b) / gg
        else:
            corr = 4 * np.pi * sp.erf(c * qq) ** 2 * a * np.exp(-gg * b) / gg * (3.0 / 5.0)
        corr[0, 0, 0] = 0.0
        k = k + corr
    return k


class MGP(WT):
    """MGP / MGPA / MGPG / MGP0 (kedf/mgp.py:15-119): the WT machinery with the MGP
    kernel at rho0 = the mean density."""

    def __init__(self, alpha=5.0 / 6.0, beta=5.0 / 6.0, maxpoint=1000, symmetrization=None, lumpfactor=0.2,
                 revke=True):
        super().__init__(alpha=alpha, beta=beta)
        self.opts = dict(maxpoints=maxpoint, symmetrization=symmetrization, lumpfactor=lumpfactor, revke=revke)

    def kernel(self, rho, grid):
        rho0 = rho.mean()
        if abs(self._saved_rho0 - rho0) > 1e-6 or rho.shape != self._shape:
            self._kernel = mgp_kernel(grid, rho0, **self.opts)
            self._saved_rho0, self._shape = rho0, rho.shape
        return self._kernel


# --------------------------------------------------------------------------
# finite-temperature Thomas-Fermi correction
# --------------------------------------------------------------------------
def ttf(rho, grid, temperature, x=1.0, old=False, calc=("E", "V")):
    """TTF (kedf/tf.py:83-204), the correction a temperature option adds to a KEDF
    ('DTTF', kedf/__init__.py:155-156): TemperatureTFPotential, TemperatureTFEnergy
    and, with temperature0 (old=True), TemperatureTFEnergy_old."""
    T = temperature
    factor = (3.0 / 10.0) * (5.0 / 3.0) * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
    vtf = factor * np.cbrt(rho * rho)
    theta = T / vtf
    c = 0.752252778063675
    mask = theta >= 1.36
    a = [0.016, -0.957, -0.293, 0.209]
    pot = np.zeros_like(theta)
    tmp = np.ones_like(theta)
    for i in range(4):
        tmp = tmp * theta
        pot += a[i] * tmp
    pot *= vtf
    t32 = 1.0 / np.sqrt(theta * theta * theta)
    pot[mask] = T * (np.log(c * t32[mask]) + np.log(1 + c * t32[mask] / 2.0 ** 1.5)) - vtf[mask]
    out = {}
    if "V" in calc:
        out["V"] = pot * x
    if "E" in calc:
        tf_ed = np.cbrt(rho * rho * rho * rho * rho) * (3.0 / 10.0) * (3.0 * np.pi ** 2) ** (2.0 / 3.0)
        if old:
            ed = (pot + vtf) * rho
            ed += -2 * np.sqrt(2) / 3 / np.pi ** 2 * T ** 2.5 / np.sqrt(theta ** 5) * np.sqrt(
                0.16 + theta * theta) / (1.0 - 0.14 * (np.exp(-theta) - np.exp(-3.68 * theta)))
            ed -= tf_ed
        else:
            b = [0.016, -0.957 * 3, -0.293 * -3, -0.209]
            k = T / factor
            ed = np.zeros_like(theta)
            tmp = rho.copy()
            for i in range(4):
                ed += b[i] * tmp
                tmp = tmp * theta
            ed *= T
            r = rho[mask]
            ed[mask] = (-2.0 * r + 2 ** 1.5 * k ** 1.5 * np.arctanh(c * t32[mask] / 2 ** 1.5) / c
                        + r * np.log(1.0 + c / 2 ** 1.5 * t32[mask]) + r * np.log(c * t32[mask])
                        + 2 ** 0.5 * k * np.sqrt(theta[mask]) * np.cbrt(r) * np.log(8.0 * k ** 3.0 - c ** 2.0 * r * r)
                        / c) * T - tf_ed[mask]
        out["E"] = ed.sum() * grid.dV * x
    return out
