// The Wang-Govind-Carter nonlocal kinetic kernel with the two-body Fermi wave
// vector (Y. A. Wang, N. Govind and E. A. Carter, Phys. Rev. B 60, 16350
// (1999)): T_NL = int int rho^alpha(r) w(xi_gamma(r, r'), r - r') rho^beta(r'),
// xi_gamma = ((k_F(r)^gamma + k_F(r')^gamma) / 2)^(1/gamma), evaluated, as the
// paper does, through the second-order Taylor expansion of the kernel about the
// Fermi wave vector k* of the average density rho0.  The reference has no
// counterpart (its density-dependent kernels are the k_F-node family,
// kedf/lwt.py).
//
// With theta = (rho - rho0) / rho0 and t = xi / k*,
//   t - 1 = (theta + theta')/6 + c1 (theta^2 + theta'^2) + c2 (theta + theta')^2 + O(theta^3),
//   c1 = (gamma/3 - 1)/12,  c2 = (1 - gamma)/72,
// and w(k* t) = K0 + K1 (t - 1) + K2 (t - 1)^2 / 2 with K1 = t dK/dt, K2 = t^2 d2K/dt2 at
// t = 1 of the Wang-Teter kernel K(q; k) = c (k/k*)^p F(q / 2k; x, 1)
// (kedf/kernel.py:325-334; c = C_TF 5/(9 alpha beta) rho0^(5/3-alpha-beta),
// p = 5 - 3(alpha + beta)):
//   K0 = c F,  K1 = c (p F - eta F'),  K2 = c (p(p-1) F + (2 - 2p) eta F' + eta^2 F'').
// To second order in theta the energy is
//   E = int a0 P0 + a1 P1 + a2 P2,   a_n = rho^alpha theta^n,  b_n = rho^beta theta^n,
//   P0 = K0*b0 + Ka*b1 + Kb*b2,  P1 = Ka*b0 + Kc*b1,  P2 = Kb*b0  (convolutions),
//   Ka = K1/6,  Kb = K1 (c1 + c2) + K2/72,  Kc = 2 (K1 c2 + K2/72),
// and its potential (rho0 held fixed, as the Wang-Teter potential holds it)
//   V = sum_n a_n' P_n + sum_n b_n' Q_n,  Q the same convolutions of the a_n.
// One evaluation: a pre-pass writing the six fields a_n, b_n, one batched R2C,
// one G-space pass forming the six products in place, one batched C2R and a
// post-pass (energy, potential).  The kernel tables K0, Ka, Kb, Kc are built on
// the device in float64 whenever rho0 moves by more than 1e-6 (the Wang-Teter
// rule, wt.py:58-73).
#include "common.cuh"
#include "pointwise.cuh"

#include <cmath>

using namespace ofdft;

namespace {

// F, eta F' and eta^2 F'' of the inverse Lindhard function (mu = 1 below), in
// the branch order of lindhard_dev: the closed form, then eta < tol, |eta - 1|
// < tol (F' capped as the reference's LindhardDerivative caps it, F'' = 0) and
// the large-eta series above 3.65 differentiated term by term.
__device__ inline void lindhard_d2(double eta, double lbda, double mu, double& F, double& eF1, double& e2F2) {
    const double tol = 1e-10, tol2 = tol / 10;
    F = eta;
    eF1 = 0.0;
    e2F2 = 0.0;
    if (eta > tol2 && fabs(eta - 1.0) > tol2) {
        const double A = log((1.0 + eta) / fabs(1.0 - eta));
        const double e2 = eta * eta;
        const double L = 0.5 + 0.25 * (1.0 - e2) * A / eta;
        const double L1 = -(1.0 + e2) * A / (4.0 * e2) + 0.5 / eta;
        const double L2 = A / (2.0 * e2 * eta) - 1.0 / (e2 * (1.0 - e2));
        F = 1.0 / L - 3.0 * mu * e2 - lbda;
        const double F1 = -L1 / (L * L) - 6.0 * mu * eta;
        const double F2 = -L2 / (L * L) + 2.0 * L1 * L1 / (L * L * L) - 6.0 * mu;
        eF1 = eta * F1;
        e2F2 = e2 * F2;
    }
    if (eta < tol) {
        const double s = 1.0 / 3.0 - 3.0 * mu;
        F = 1.0 - lbda + eta * eta * s;
        eF1 = 2.0 * eta * eta * s;
        e2F2 = 2.0 * eta * eta * s;
    }
    if (fabs(eta - 1.0) < tol) {
        F = 2.0 - lbda - 3.0 * mu + 20.0 * (eta - 1.0);
        eF1 = 48.0 * eta;
        e2F2 = 0.0;
    }
    if (eta > 3.65) {
        const double c[15] = {-0.13714285714285712, -6.39999999999999875e-2, -3.77825602968460128e-2,
                              -2.51824061652633074e-2, -1.80879839616166146e-2, -1.36715733124818332e-2,
                              -1.07236045520990083e-2, -8.65192783339199453e-3, -7.1372762502456763e-3,
                              -5.9945117538835746e-3, -5.10997527675418131e-3, -4.41060829979912465e-3,
                              -3.84763737842981233e-3, -3.38745061493813488e-3, -3.00624946457977689e-3};
        const double inv2 = 1.0 / (eta * eta);
        double f = 0.0, d1 = 0.0, d2 = 0.0, pw = inv2;
        for (int k = 0; k < 15; ++k) {
            const double m = 2.0 * (k + 1);  // eta^-m
            f += c[k] * pw;
            d1 += -m * c[k] * pw;
            d2 += m * (m + 1.0) * c[k] * pw;
            pw *= inv2;
        }
        F = 3.0 * (1.0 - mu) * eta * eta - lbda - 0.6 + f;
        eF1 = 6.0 * (1.0 - mu) * eta * eta + d1;
        e2F2 = 6.0 * (1.0 - mu) * eta * eta + d2;
    }
}

struct WgcCoef {
    double c, p, tkf, x;   // prefactor, exponent, 2 k*, TF share of the Lindhard function
    double ka, kb1, kb2, kc1, kc2;  // Ka = ka K1; Kb = kb1 K1 + kb2 K2; Kc = kc1 K1 + kc2 K2
};

// K0, Ka, Kb, Kc per half-grid point (grid precision), K(G = 0) = 0
template <typename T>
__global__ void k_wgc_tables(T* tab, Geo geo, WgcCoef w) {
    const long long Nc = geo.Nc;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < Nc; i += stride) {
        const double q = sqrt(gsq(geo, i));
        double F, eF1, e2F2;
        lindhard_d2(q / w.tkf, w.x, 1.0, F, eF1, e2F2);
        const double K0 = w.c * F;
        const double K1 = w.c * (w.p * F - eF1);
        const double K2 = w.c * (w.p * (w.p - 1.0) * F + (2.0 - 2.0 * w.p) * eF1 + e2F2);
        const bool g0 = i == 0;
        tab[i] = g0 ? (T)0 : (T)K0;
        tab[Nc + i] = g0 ? (T)0 : (T)(w.ka * K1);
        tab[2 * Nc + i] = g0 ? (T)0 : (T)(w.kb1 * K1 + w.kb2 * K2);
        tab[3 * Nc + i] = g0 ? (T)0 : (T)(w.kc1 * K1 + w.kc2 * K2);
    }
}

// a0, a1, a2, b0, b1, b2 (fields 0..5 of f, N apart)
template <typename T>
__global__ void k_wgc_pre(const T* __restrict__ rho, T* f, long long N, T alpha, T beta, T rho0, T inv_rho0) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const T r = rho[i];
        const T rc = r < (T)kZERO ? (T)kZERO : r;  // wt.py's clamp of the powers
        const T th = (r - rho0) * inv_rho0;
        const T ra = mpow(rc, alpha), rb = mpow(rc, beta);
        f[i] = ra;
        f[N + i] = ra * th;
        f[2 * N + i] = ra * th * th;
        f[3 * N + i] = rb;
        f[4 * N + i] = rb * th;
        f[5 * N + i] = rb * th * th;
    }
}

// the six products in place: slots 0..2 <- P0..P2 (from the b's), 3..5 <- Q0..Q2 (from the a's)
template <typename T>
__global__ void k_wgc_gspace(typename Cplx<T>::type* S, const T* __restrict__ tab, long long Nc, T invN) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < Nc; i += stride) {
        const T K0 = tab[i] * invN, Ka = tab[Nc + i] * invN, Kb = tab[2 * Nc + i] * invN, Kc = tab[3 * Nc + i] * invN;
        const auto a0 = S[i], a1 = S[Nc + i], a2 = S[2 * Nc + i];
        const auto b0 = S[3 * Nc + i], b1 = S[4 * Nc + i], b2 = S[5 * Nc + i];
        auto lin3 = [](T k0, decltype(a0) x0, T k1, decltype(a0) x1, T k2, decltype(a0) x2) {
            auto z = x0;
            z.x = k0 * x0.x + k1 * x1.x + k2 * x2.x;
            z.y = k0 * x0.y + k1 * x1.y + k2 * x2.y;
            return z;
        };
        S[i] = lin3(K0, b0, Ka, b1, Kb, b2);
        S[Nc + i] = lin3(Ka, b0, Kc, b1, (T)0, b2);
        S[2 * Nc + i] = lin3(Kb, b0, (T)0, b1, (T)0, b2);
        S[3 * Nc + i] = lin3(K0, a0, Ka, a1, Kb, a2);
        S[4 * Nc + i] = lin3(Ka, a0, Kc, a1, (T)0, a2);
        S[5 * Nc + i] = lin3(Kb, a0, (T)0, a1, (T)0, a2);
    }
}

// energy density a0 P0 + a1 P1 + a2 P2 (block partials) and the potential
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_wgc_post(const T* __restrict__ rho, const T* __restrict__ P, T* V,
                                                          long long N, T alpha, T beta, T rho0, T inv_rho0,
                                                          double* partials) {
    RunSum<T> sum;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const T r = rho[i];
        const T rc = r < (T)kZERO ? (T)kZERO : r;
        const T th = (r - rho0) * inv_rho0;
        const T ra = mpow(rc, alpha), rb = mpow(rc, beta);
        const T P0 = P[i], P1 = P[N + i], P2 = P[2 * N + i];
        const T Q0 = P[3 * N + i], Q1 = P[4 * N + i], Q2 = P[5 * N + i];
        sum.add(ra * (P0 + th * (P1 + th * P2)));
        if (V) {
            // d(rho^s theta^n)/drho = s rho^(s-1) theta^n + rho^s n theta^(n-1) / rho0
            const T da = alpha * ra / rc, db = beta * rb / rc;
            const T va = da * (P0 + th * (P1 + th * P2)) + ra * inv_rho0 * (P1 + (T)2 * th * P2);
            const T vb = db * (Q0 + th * (Q1 + th * Q2)) + rb * inv_rho0 * (Q1 + (T)2 * th * Q2);
            V[i] = va + vb;
        }
    }
    double acc[1] = {sum.get()};
    block_sum_store<1>(acc, partials);
}

}  // namespace

struct ofdft_wgc {
    ofdft_grid* g = nullptr;
    double alpha = 0, beta = 0, gamma = 0, x = 1, rho0_user = 0;
    double rho0_tab = -1.0;  // rho0 of the current tables
    double* h_res = nullptr;  // pinned
    Scratch sc;
    ~ofdft_wgc() { cudaFreeHost(h_res); }
};

namespace {

template <typename T>
void wgc_compute_t(ofdft_wgc* w, const T* rho, T* V, unsigned calc, double* energy, cudaStream_t st) {
    using C = typename Cplx<T>::type;
    ofdft_grid* g = w->g;
    const long long N = g->N, Nc = g->Nc;
    double rho0 = w->rho0_user;
    if (!(rho0 > 0.0)) {  // the mean density of this call (wt.py:112-113)
        double s = 0.0;
        const int rc = ofdft_dot(g, rho, nullptr, &s, (ofdft_stream)st);
        OFDFT_REQUIRE(rc == OFDFT_OK, "WGC kernel: %s", ofdft_last_error());
        rho0 = s / (double)N;
    }
    OFDFT_REQUIRE(rho0 > 0.0, "WGC kernel: the reference density rho0 must be positive");
    T* tab = (T*)w->sc.get("tab", 4 * (size_t)Nc * sizeof(T));
    const int eb = blocks_for(N, 256, g->sms * 16), gb = blocks_for(Nc, 256, g->sms * 16);
    if (w->rho0_tab < 0.0 || std::fabs(rho0 - w->rho0_tab) > 1e-6) {
        const double pi = M_PI;
        const double cTF = 0.3 * std::pow(3.0 * pi * pi, 2.0 / 3.0);
        WgcCoef c;
        c.c = 5.0 / (9.0 * w->alpha * w->beta * std::pow(rho0, w->alpha + w->beta - 5.0 / 3.0)) * cTF;
        c.p = 5.0 - 3.0 * (w->alpha + w->beta);
        c.tkf = 2.0 * std::cbrt(3.0 * rho0 * pi * pi);
        c.x = w->x;
        const double c1 = (w->gamma / 3.0 - 1.0) / 12.0, c2 = (1.0 - w->gamma) / 72.0;
        c.ka = 1.0 / 6.0;
        c.kb1 = c1 + c2;
        c.kb2 = 1.0 / 72.0;
        c.kc1 = 2.0 * c2;
        c.kc2 = 2.0 / 72.0;
        k_wgc_tables<T><<<gb, 256, 0, st>>>(tab, g->geo, c);
        OFDFT_LAUNCH_CHECK();
        w->rho0_tab = rho0;
    }
    T* f = (T*)w->sc.get("fields", 6 * (size_t)N * sizeof(T));
    C* S = (C*)w->sc.get("spectra", 6 * (size_t)Nc * sizeof(C));
    const T a = (T)w->alpha, b = (T)w->beta, r0 = (T)rho0, ir0 = (T)(1.0 / rho0);
    k_wgc_pre<T><<<eb, 256, 0, st>>>(rho, f, N, a, b, r0, ir0);
    OFDFT_LAUNCH_CHECK();
    g->exec_r2c(f, S, 6, st);
    k_wgc_gspace<T><<<gb, 256, 0, st>>>(S, tab, Nc, (T)(1.0 / (double)N));
    OFDFT_LAUNCH_CHECK();
    g->exec_c2r(S, f, 6, st);
    k_wgc_post<T><<<g->red_blocks, RED_THREADS, 0, st>>>(rho, f, (calc & OFDFT_CALC_V) ? V : nullptr, N, a, b, r0,
                                                          ir0, g->d_partials);
    OFDFT_LAUNCH_CHECK();
    reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 1, 0ull, g->d_results);
    OFDFT_LAUNCH_CHECK();
    OFDFT_CK(cudaMemcpyAsync(w->h_res, g->d_results, sizeof(double), cudaMemcpyDeviceToHost, st));
    OFDFT_CK(cudaStreamSynchronize(st));
    if (energy) *energy = w->h_res[0] * g->dV;
}

}  // namespace

extern "C" {

int ofdft_wgc_create(ofdft_grid* g, double alpha, double beta, double gamma, double x, double rho0,
                     ofdft_wgc** out) {
    return guard([&] {
        OFDFT_REQUIRE(g && out, "ofdft_wgc_create: null argument");
        OFDFT_REQUIRE(alpha > 0.0 && beta > 0.0 && gamma > 0.0, "ofdft_wgc_create: alpha, beta, gamma must be > 0");
        auto* w = new ofdft_wgc();
        w->g = g;
        w->alpha = alpha;
        w->beta = beta;
        w->gamma = gamma;
        w->x = x;
        w->rho0_user = rho0;
        cudaError_t e = cudaMallocHost(&w->h_res, sizeof(double));
        if (e != cudaSuccess) {
            delete w;
            OFDFT_CK(e);
        }
        *out = w;
    });
}

int ofdft_wgc_compute(ofdft_wgc* w, const void* rho, void* v_out, unsigned calc, double* energy, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(w && rho, "ofdft_wgc_compute: null argument");
        OFDFT_REQUIRE(!(calc & OFDFT_CALC_V) || v_out, "ofdft_wgc_compute: V requested but v_out is NULL");
        if (w->g->prec == OFDFT_F64)
            wgc_compute_t<double>(w, (const double*)rho, (double*)v_out, calc, energy, (cudaStream_t)s);
        else
            wgc_compute_t<float>(w, (const float*)rho, (float*)v_out, calc, energy, (cudaStream_t)s);
    });
}

void ofdft_wgc_destroy(ofdft_wgc* w) { delete w; }

}  // extern "C"
