// Local pseudopotential on the grid (LocalPseudo, src/dftpy/functional/pseudo/
// __init__.py:74-452, :505-571): radial v_loc(q) lines from not-a-knot cubic
// splines of the tabulated potential, the structure factor by smooth PME
// (B-spline spreading + R2C) or exactly, and the forces of both paths.
#include "common.cuh"
#include "host_math.h"
#include "pme.cuh"

#include <algorithm>
#include <cstring>

using namespace ofdft;

namespace {

constexpr int kMaxSpecies = 16;

// device view of one species' radial line
struct Line {
    const double* x;   // spline knots gp[1:]
    const double* c;   // 4 coefficients per interval
    int n;             // number of knots
    double gp1, gplast, dp;
    double v0, v1, v2;  // vp[0..2] for the quartic near q = 0
};

struct Lines {
    Line s[kMaxSpecies];
    int ns;
};

// LocalPseudo.calc_vlines (pseudo/__init__.py:398-423)
__device__ inline double vline_eval(const Line& L, double q) {
    if (q < L.gp1) {
        // quartic_interpolation of [v2, v1, v0, v1, v2] at q/dp (math_utils.py:390-400)
        const double f0 = L.v2, f1 = L.v1, f2 = L.v0, f3 = L.v1, f4 = L.v2;
        const double t0 = f2;
        const double t1 = 2.0 * f0 - 16.0 * f1 + 16.0 * f3 - 2.0 * f4;
        const double t2 = -f0 + 16.0 * f1 - 30.0 * f2 + 16.0 * f3 - f4;
        const double t3 = -2.0 * f0 + 4.0 * f1 - 4.0 * f3 + 2.0 * f4;
        const double t4 = f0 - 4.0 * f1 + 6.0 * f2 - 4.0 * f3 + f4;
        const double dx = q / L.dp;
        return t0 + dx * (t1 + dx * (t2 + dx * (t3 + dx * t4))) / 24.0;
    }
    if (q < L.gplast) {
        int lo = 0, hi = L.n - 1;  // largest i with x[i] <= q, clamped to [0, n-2]
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (L.x[mid] <= q) lo = mid;
            else hi = mid;
        }
        double u = q - L.x[lo];
        const double* c = L.c + 4 * (long long)lo;
        return c[0] + u * (c[1] + u * (c[2] + u * c[3]));
    }
    return 0.0;
}

// v(G) (+)= vline_s(|G|) * F(G) * B(G) * scale   (PME, _PP_Reciprocal_PME :437-452)
template <typename T>
__global__ void k_pp_accum_pme(const typename Cplx<T>::type* __restrict__ QG, typename Cplx<T>::type* vG, Line L,
                               const double* bre, const double* bim, int first, Geo geo, double scale) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        double q = sqrt(gsq(geo, i));
        double vl = vline_eval(L, q);
        double br, bi;
        barray(bre, bim, geo, i, br, bi);
        double qr = (double)QG[i].x, qi = (double)QG[i].y;
        double xr = vl * (qr * br - qi * bi) * scale;
        double xi = vl * (qr * bi + qi * br) * scale;
        if (!first) {
            xr += (double)vG[i].x;
            xi += (double)vG[i].y;
        }
        vG[i].x = (T)xr;
        vG[i].y = (T)xi;
    }
}

// exact structure factor: v(G) = sum_a vline_{s(a)}(|G|) exp(-i G.R_a) * scale  (:425-435)
template <typename T>
__global__ void k_pp_exact(typename Cplx<T>::type* vG, Lines LS, const double* __restrict__ pos,
                           const int* __restrict__ spec, int nat, Geo geo, double scale) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        double q = sqrt(gg);
        double vl[kMaxSpecies];
        for (int s = 0; s < LS.ns; ++s) vl[s] = vline_eval(LS.s[s], q);
        double sr = 0.0, si = 0.0;
        for (int a = 0; a < nat; ++a) {
            double ph = gx * pos[3 * a] + gy * pos[3 * a + 1] + gz * pos[3 * a + 2];
            double sn, cs;
            sincos(ph, &sn, &cs);
            sr += vl[spec[a]] * cs;
            si -= vl[spec[a]] * sn;
        }
        vG[i].x = (T)(sr * scale);
        vG[i].y = (T)(si * scale);
    }
}

// rho(G) conj(B(G)) vline_s(|G|) / N with G = 0 removed (_ForcePME :527-536)
template <typename T>
__global__ void k_pp_force_pme(const typename Cplx<T>::type* __restrict__ rhoG, typename Cplx<T>::type* out, Line L,
                               const double* bre, const double* bim, Geo geo, double scale) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        double q = sqrt(gsq(geo, i));
        double vl = vline_eval(L, q);
        double br, bi;
        barray(bre, bim, geo, i, br, bi);
        double qr = (double)rhoG[i].x, qi = (double)rhoG[i].y;
        double xr = vl * (qr * br + qi * bi) * scale;   // rho * conj(B)
        double xi = vl * (qi * br - qr * bi) * scale;
        if (i == 0) xr = xi = 0.0;
        out[i].x = (T)xr;
        out[i].y = (T)xi;
    }
}

// exact forces (_Force :505-521): F_a = 2/V sum_{G in mask} G vline Im(rho(G) e^{i G.R_a});
// one chunk of up to 8 atoms per launch, block partials of 3 x chunk sums.
constexpr int kForceChunk = 8;

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pp_force_exact(const typename Cplx<T>::type* __restrict__ rhoG,
                                                                  Lines LS, const double* __restrict__ pos,
                                                                  const int* __restrict__ spec, int a0, int na,
                                                                  Geo geo, double rscale, double* partials) {
    double acc[3 * kForceChunk];
    for (int t = 0; t < 3 * kForceChunk; ++t) acc[t] = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        if (!half_mask(geo, i)) continue;
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        double q = sqrt(gg);
        double rr = (double)rhoG[i].x * rscale, ri = (double)rhoG[i].y * rscale;
        for (int t = 0; t < na; ++t) {
            const int a = a0 + t;
            double ph = gx * pos[3 * a] + gy * pos[3 * a + 1] + gz * pos[3 * a + 2];
            double sn, cs;
            sincos(ph, &sn, &cs);
            double den = vline_eval(LS.s[spec[a]], q) * (rr * sn + ri * cs);  // Im(rho e^{i ph})
            acc[3 * t + 0] += gx * den;
            acc[3 * t + 1] += gy * den;
            acc[3 * t + 2] += gz * den;
        }
    }
    block_sum_store<3 * kForceChunk>(acc, partials);
}

// Gradient of E_PP = int v_loc rho dV with respect to the radial table of each
// species.  E_PP = (dV/V) sum_{G in half grid} w_G vline_s(|G|) Re(S_s(G) conj(rho(G)))
// (w_G = 2 off the k2 = 0 / Nyquist planes, 1 on them), and vline is linear in
// the table: a quartic in vp[0..2] below gp[1], a cubic spline of vp[1:] above.
// Per G this kernel adds h = (dV/V) w_G Re(S conj rho) times the derivative of
// vline with respect to the quartic's three values, or times u^p (p = 0..3) to
// the spline interval holding |G|; the host applies the spline adjoint.
template <typename T>
__global__ void k_pp_grad_moments(const typename Cplx<T>::type* __restrict__ rhoG,
                                  const typename Cplx<T>::type* __restrict__ QG, const double* bre,
                                  const double* bim, Line L, Geo geo, double scale, double* moments,
                                  double* quart) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        double q = sqrt(gsq(geo, i));
        if (q >= L.gplast) continue;
        double br = 1.0, bi = 0.0;  // no B-spline factor for exact structure factors
        if (bre) barray(bre, bim, geo, i, br, bi);
        const double qr = (double)QG[i].x, qi = (double)QG[i].y;
        const double sr = qr * br - qi * bi, si = qr * bi + qi * br;
        const int k2 = (int)(i % geo.n2h);
        const double w = (k2 == 0 || (geo.n2 % 2 == 0 && k2 == geo.n2 / 2)) ? 1.0 : 2.0;
        const double h = scale * w * (sr * (double)rhoG[i].x + si * (double)rhoG[i].y);
        if (q < L.gp1) {
            const double dx = q / L.dp, x2 = dx * dx, x4 = x2 * x2;
            atomicAdd(&quart[0], (1.0 + (-30.0 * x2 + 6.0 * x4) / 24.0) * h);
            atomicAdd(&quart[1], ((32.0 * x2 - 8.0 * x4) / 24.0) * h);
            atomicAdd(&quart[2], ((-2.0 * x2 + 2.0 * x4) / 24.0) * h);
            continue;
        }
        int lo = 0, hi = L.n - 1;
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (L.x[mid] <= q) lo = mid;
            else hi = mid;
        }
        const double u = q - L.x[lo];
        double* mp = moments + 4 * (long long)lo;
        atomicAdd(&mp[0], h);
        atomicAdd(&mp[1], h * u);
        atomicAdd(&mp[2], h * u * u);
        atomicAdd(&mp[3], h * u * u * u);
    }
}

// dv_s/dq: the derivative of the species' spline (splev der=1) below max(gp),
// 0 above (_PP_Derivative_One, pseudo/__init__.py:454-460).  Unlike the
// potential lines this uses the spline down to q = 0 (its first piece extended
// below gp[1]); the quartic near q = 0 is not differentiated.
__device__ inline double vline_deriv(const Line& L, double q) {
    if (!(q < L.gplast)) return 0.0;
    int lo = 0, hi = L.n - 1;  // largest i with x[i] <= q, clamped to [0, n-2]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (L.x[mid] <= q) lo = mid;
        else hi = mid;
    }
    const double u = q - L.x[lo];
    const double* c = L.c + 4 * (long long)lo;
    return c[1] + u * (2.0 * c[2] + u * 3.0 * c[3]);
}

__device__ __forceinline__ void sym6(double gx, double gy, double gz, double (&t)[6]) {
    t[0] = gx * gx;
    t[1] = gx * gy;
    t[2] = gx * gz;
    t[3] = gy * gy;
    t[4] = gy * gz;
    t[5] = gz * gz;
}

// PME stress sums of one species over the mask (_StressPME :590-600, raw
// transforms): g_i g_j Re(conj(rho(G)) B(G) Q_s(G)) v_s'(|G|) / |G|
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pp_stress_pme(const typename Cplx<T>::type* __restrict__ rhoG,
                                                               const typename Cplx<T>::type* __restrict__ QG, Line L,
                                                               const double* bre, const double* bim, Geo geo,
                                                               double* partials) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        if (!half_mask(geo, i)) continue;
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        const double q = sqrt(gg);
        const double invq = (i == 0) ? 0.0 : 1.0 / q;
        double br, bi;
        barray(bre, bim, geo, i, br, bi);
        const double rr = (double)rhoG[i].x, ri = (double)rhoG[i].y;
        const double xr = rr * br + ri * bi, xi = rr * bi - ri * br;  // conj(rho) B
        const double re = (xr * (double)QG[i].x - xi * (double)QG[i].y) * vline_deriv(L, q) * invq;
        double t[6];
        sym6(gx, gy, gz, t);
        for (int k = 0; k < 6; ++k) acc[k] += t[k] * re;
    }
    block_sum_store<6>(acc, partials);
}

// exact stress sums over the mask (_Stress :479-503, _PP_Derivative :462-477):
// g_i g_j Re(rho(G) sum_a v_{s(a)}'(|G|) e^{i G.R_a}) / |G|
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pp_stress_exact(const typename Cplx<T>::type* __restrict__ rhoG,
                                                                 Lines LS, const double* __restrict__ pos,
                                                                 const int* __restrict__ spec, int nat, Geo geo,
                                                                 double* partials) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        if (!half_mask(geo, i)) continue;
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        const double q = sqrt(gg);
        const double invq = (i == 0) ? 0.0 : 1.0 / q;
        double dv[kMaxSpecies];
        for (int s = 0; s < LS.ns; ++s) dv[s] = vline_deriv(LS.s[s], q);
        double vr = 0.0, vi = 0.0;
        for (int a = 0; a < nat; ++a) {
            const double ph = gx * pos[3 * a] + gy * pos[3 * a + 1] + gz * pos[3 * a + 2];
            double sn, cs;
            sincos(ph, &sn, &cs);
            vr += dv[spec[a]] * cs;
            vi += dv[spec[a]] * sn;
        }
        const double re = ((double)rhoG[i].x * vr - (double)rhoG[i].y * vi) * invq;
        double t[6];
        sym6(gx, gy, gz, t);
        for (int k = 0; k < 6; ++k) acc[k] += t[k] * re;
    }
    block_sum_store<6>(acc, partials);
}

// exact structure factor of one species, S_s(G) = sum_{a in s} exp(-i G.R_a), as a complex field
template <typename T>
__global__ void k_strf_species(typename Cplx<T>::type* S, const double* __restrict__ pos, const int* __restrict__ sel,
                               int na, Geo geo) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        double sr = 0.0, si = 0.0;
        for (int t = 0; t < na; ++t) {
            const int a = sel[t];
            double ph = gx * pos[3 * a] + gy * pos[3 * a + 1] + gz * pos[3 * a + 2];
            double sn, cs;
            sincos(ph, &sn, &cs);
            sr += cs;
            si -= sn;
        }
        S[i].x = (T)sr;
        S[i].y = (T)si;
    }
}

}  // namespace

struct ofdft_pseudo {
    ofdft_grid* g = nullptr;
    int ns = 0, pme = 1, order = 10;
    std::vector<CubicSpline> spl;
    std::vector<double> gp1, gplast, dp, v0, v1, v2;
    std::vector<double*> d_x, d_c;
    std::vector<int> npts;
    // ions
    int nat = 0;
    std::vector<double> pos, frac;
    std::vector<int> spec;
    double* d_pos = nullptr;
    double* d_frac = nullptr;
    int* d_spec = nullptr;
    int* d_sel = nullptr;         // atom indices grouped by species
    std::vector<int> sel_off;     // species offsets into d_sel
    double* d_bre = nullptr;      // B-spline Euler factors, axes packed
    double* d_bim = nullptr;
    double* d_cinv = nullptr;     // inv(lattice), row-major
    double* d_scale = nullptr;    // per-atom gather scale
    std::vector<ofdft::PmeTiles> tiles;  // deterministic spreading work list per species (PME)
    Scratch sc;

    Line line(int s) const {
        Line L;
        L.x = d_x[s];
        L.c = d_c[s];
        L.n = (int)spl[s].x.size();
        L.gp1 = gp1[s];
        L.gplast = gplast[s];
        L.dp = dp[s];
        L.v0 = v0[s];
        L.v1 = v1[s];
        L.v2 = v2[s];
        return L;
    }
    Lines lines() const {
        Lines LS;
        LS.ns = ns;
        for (int s = 0; s < ns; ++s) LS.s[s] = line(s);
        return LS;
    }
};

namespace ofdft {
// fractional coordinates wrapped to [0, 1) (ase get_scaled_positions(wrap=True))
void frac_coords(const double* lattice, int nat, const double* pos, std::vector<double>& frac) {
    const double* a = lattice;
    double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) + a[2] * (a[3] * a[7] - a[4] * a[6]);
    double inv[9];
    inv[0] = (a[4] * a[8] - a[5] * a[7]) / det;
    inv[1] = (a[2] * a[7] - a[1] * a[8]) / det;
    inv[2] = (a[1] * a[5] - a[2] * a[4]) / det;
    inv[3] = (a[5] * a[6] - a[3] * a[8]) / det;
    inv[4] = (a[0] * a[8] - a[2] * a[6]) / det;
    inv[5] = (a[2] * a[3] - a[0] * a[5]) / det;
    inv[6] = (a[3] * a[7] - a[4] * a[6]) / det;
    inv[7] = (a[1] * a[6] - a[0] * a[7]) / det;
    inv[8] = (a[0] * a[4] - a[1] * a[3]) / det;
    frac.resize(3 * (size_t)nat);
    for (int i = 0; i < nat; ++i) {
        for (int d = 0; d < 3; ++d) {
            double f = pos[3 * i] * inv[0 + d] + pos[3 * i + 1] * inv[3 + d] + pos[3 * i + 2] * inv[6 + d];
            f = std::fmod(f, 1.0);
            if (f < 0) f += 1.0;
            if (f >= 1.0) f = 0.0;
            frac[3 * i + d] = f;
        }
    }
}

void lattice_inverse(const double* a, double* inv) {
    double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) + a[2] * (a[3] * a[7] - a[4] * a[6]);
    inv[0] = (a[4] * a[8] - a[5] * a[7]) / det;
    inv[1] = (a[2] * a[7] - a[1] * a[8]) / det;
    inv[2] = (a[1] * a[5] - a[2] * a[4]) / det;
    inv[3] = (a[5] * a[6] - a[3] * a[8]) / det;
    inv[4] = (a[0] * a[8] - a[2] * a[6]) / det;
    inv[5] = (a[2] * a[3] - a[0] * a[5]) / det;
    inv[6] = (a[3] * a[7] - a[4] * a[6]) / det;
    inv[7] = (a[1] * a[6] - a[0] * a[7]) / det;
    inv[8] = (a[0] * a[4] - a[1] * a[3]) / det;
}

// per-axis B-spline Euler factor tables packed [axis0 | axis1 | axis2(half)]
void bspline_tables(const ofdft_grid* g, int order, double** d_re, double** d_im) {
    std::vector<double> re, im, r, i;
    for (int d = 0; d < 3; ++d) {
        int nG = d == 2 ? g->n2h : g->nr[d];
        bspline_bm(g->nr[d], nG, order, r, i);
        re.insert(re.end(), r.begin(), r.end());
        im.insert(im.end(), i.begin(), i.end());
    }
    OFDFT_CK(cudaMalloc(d_re, re.size() * sizeof(double)));
    OFDFT_CK(cudaMalloc(d_im, im.size() * sizeof(double)));
    upload_now(*d_re, re.data(), re.size() * sizeof(double));
    upload_now(*d_im, im.data(), im.size() * sizeof(double));
}
}  // namespace ofdft

namespace {

template <typename T>
void vloc_t(ofdft_pseudo* p, T* out, cudaStream_t st) {
    ofdft_grid* g = p->g;
    using C = typename Cplx<T>::type;
    const size_t cb = g->cplx_bytes(), rb = g->real_bytes();
    C* vG = (C*)p->sc.get("vG", cb);
    const int gblk = blocks_for(g->Nc, 256, g->sms * 16);
    const double scale = 1.0 / g->volume;  // irfftn(v)/dV = raw/(N dV)
    if (p->pme) {
        T* Q = (T*)p->sc.get("Q", rb);
        C* QG = (C*)p->sc.get("QG", cb);
        bool first = true;
        for (int s = 0; s < p->ns; ++s) {
            const int n_s = p->sel_off[s + 1] - p->sel_off[s];
            if (n_s > 0) pme_spread<T>(p->tiles[s], p->d_frac, p->d_sel + p->sel_off[s], nullptr, g->geo, Q, rb, st);
            else OFDFT_CK(cudaMemsetAsync(Q, 0, rb, st));
            g->exec_r2c(Q, QG, 1, st);
            k_pp_accum_pme<T><<<gblk, 256, 0, st>>>(QG, vG, p->line(s), p->d_bre, p->d_bim, first, g->geo, scale);
            OFDFT_LAUNCH_CHECK();
            first = false;
        }
    } else {
        k_pp_exact<T><<<gblk, 256, 0, st>>>(vG, p->lines(), p->d_pos, p->d_spec, p->nat, g->geo, scale);
        OFDFT_LAUNCH_CHECK();
    }
    g->exec_c2r(vG, out, 1, st);
}

template <typename T>
void forces_t(ofdft_pseudo* p, const T* rho, double* F, cudaStream_t st) {
    ofdft_grid* g = p->g;
    using C = typename Cplx<T>::type;
    const size_t cb = g->cplx_bytes(), rb = g->real_bytes();
    C* rhoG = (C*)p->sc.get("rhoG", cb);
    g->exec_r2c(rho, rhoG, 1, st);
    const int gblk = blocks_for(g->Nc, 256, g->sms * 16);
    double* dF = (double*)p->sc.get("F", 3 * (size_t)std::max(1, p->nat) * sizeof(double));
    if (p->pme) {
        C* X = (C*)p->sc.get("X", cb);
        T* rhoPB = (T*)p->sc.get("rhoPB", rb);
        for (int s = 0; s < p->ns; ++s) {
            const int n_s = p->sel_off[s + 1] - p->sel_off[s];
            if (n_s == 0) continue;
            k_pp_force_pme<T><<<gblk, 256, 0, st>>>(rhoG, X, p->line(s), p->d_bre, p->d_bim, g->geo,
                                                    1.0 / (double)g->N);
            OFDFT_LAUNCH_CHECK();
            g->exec_c2r(X, rhoPB, 1, st);
            k_pme_gather<T><<<n_s, 256, 0, st>>>(p->d_frac, p->d_sel + p->sel_off[s], p->order, g->geo, rhoPB,
                                                 p->d_cinv, p->d_scale, dF);
            OFDFT_LAUNCH_CHECK();
        }
        OFDFT_CK(cudaMemcpyAsync(F, dF, 3 * (size_t)p->nat * sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
    } else {
        const double rscale = g->dV;
        std::vector<double> h(3 * kForceChunk);
        for (int a0 = 0; a0 < p->nat; a0 += kForceChunk) {
            const int na = std::min(kForceChunk, p->nat - a0);
            k_pp_force_exact<T><<<g->red_blocks, RED_THREADS, 0, st>>>(rhoG, p->lines(), p->d_pos, p->d_spec, a0, na,
                                                                       g->geo, rscale, g->d_partials);
            OFDFT_LAUNCH_CHECK();
            reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 3 * kForceChunk, 0ull,
                                                       g->d_results);
            OFDFT_LAUNCH_CHECK();
            OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, 3 * kForceChunk * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
            OFDFT_CK(cudaStreamSynchronize(st));
            for (int t = 0; t < na; ++t)
                for (int c = 0; c < 3; ++c) F[3 * (a0 + t) + c] = g->h_results[3 * t + c] * 2.0 / g->volume;
        }
    }
}

template <typename T>
void stress_t(ofdft_pseudo* p, const T* rho, double energy, double* S, cudaStream_t st) {
    ofdft_grid* g = p->g;
    using C = typename Cplx<T>::type;
    const size_t cb = g->cplx_bytes(), rb = g->real_bytes();
    const double V = g->volume, dV = g->dV;
    if (std::isnan(energy)) {  // E_PP = int v_loc rho dV (LocalPseudo.__call__)
        T* v = (T*)p->sc.get("st_v", rb);
        vloc_t<T>(p, v, st);
        double d = 0.0;
        const int rc = ofdft_dot(g, v, rho, &d, st);
        if (rc != OFDFT_OK) throw Error{rc};
        energy = d * dV;
    }
    C* rhoG = (C*)p->sc.get("rhoG", cb);
    g->exec_r2c(rho, rhoG, 1, st);
    double sum6[6] = {0, 0, 0, 0, 0, 0};
    auto fetch6 = [&] {
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 6, 0ull, g->d_results);
        OFDFT_LAUNCH_CHECK();
        OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        for (int k = 0; k < 6; ++k) sum6[k] += g->h_results[k];
    };
    double scale;
    if (p->pme) {
        T* Q = (T*)p->sc.get("Q", rb);
        C* QG = (C*)p->sc.get("QG", cb);
        for (int s = 0; s < p->ns; ++s) {
            const int n_s = p->sel_off[s + 1] - p->sel_off[s];
            if (n_s == 0) continue;
            pme_spread<T>(p->tiles[s], p->d_frac, p->d_sel + p->sel_off[s], nullptr, g->geo, Q, rb, st);
            g->exec_r2c(Q, QG, 1, st);
            k_pp_stress_pme<T><<<g->red_blocks, RED_THREADS, 0, st>>>(rhoG, QG, p->line(s), p->d_bre, p->d_bim,
                                                                      g->geo, g->d_partials);
            OFDFT_LAUNCH_CHECK();
            fetch6();
        }
        // rho and Q in the reference carry dV each; times 2 nnrR, over V^2 (:598-603)
        scale = -2.0 * (double)g->N * dV * dV / (V * V);
    } else {
        k_pp_stress_exact<T><<<g->red_blocks, RED_THREADS, 0, st>>>(rhoG, p->lines(), p->d_pos, p->d_spec, p->nat,
                                                                    g->geo, g->d_partials);
        OFDFT_LAUNCH_CHECK();
        fetch6();
        scale = -2.0 * dV / V;  // rho carries dV; -2/V (:498-499)
    }
    static const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {0, 1, 2, 1, 2, 2};
    for (int k = 0; k < 6; ++k) S[3 * I[k] + J[k]] = S[3 * J[k] + I[k]] = sum6[k] * scale;
    for (int d = 0; d < 3; ++d) S[4 * d] -= energy;
    for (int k = 0; k < 9; ++k) S[k] /= V;
}

template <typename T>
void vloc_grad_t(ofdft_pseudo* p, const T* rho, double* grad, cudaStream_t st) {
    ofdft_grid* g = p->g;
    using C = typename Cplx<T>::type;
    const size_t cb = g->cplx_bytes(), rb = g->real_bytes();
    C* rhoG = (C*)p->sc.get("rhoG", cb);
    C* SG = (C*)p->sc.get("QG", cb);
    g->exec_r2c(rho, rhoG, 1, st);
    const int gblk = blocks_for(g->Nc, 256, g->sms * 16);
    const double scale = g->dV / g->volume;
    size_t off = 0;
    for (int s = 0; s < p->ns; ++s) {
        const int n_s = p->sel_off[s + 1] - p->sel_off[s];
        const int nint = (int)p->spl[s].x.size() - 1;
        double* mom = (double*)p->sc.get("mom", (4 * (size_t)nint + 3) * sizeof(double));
        OFDFT_CK(cudaMemsetAsync(mom, 0, (4 * (size_t)nint + 3) * sizeof(double), st));
        if (n_s > 0) {
            if (p->pme) {
                T* Q = (T*)p->sc.get("Q", rb);
                pme_spread<T>(p->tiles[s], p->d_frac, p->d_sel + p->sel_off[s], nullptr, g->geo, Q, rb, st);
                g->exec_r2c(Q, SG, 1, st);
                k_pp_grad_moments<T><<<gblk, 256, 0, st>>>(rhoG, SG, p->d_bre, p->d_bim, p->line(s), g->geo, scale,
                                                           mom, mom + 4 * (size_t)nint);
            } else {
                k_strf_species<T><<<gblk, 256, 0, st>>>(SG, p->d_pos, p->d_sel + p->sel_off[s], n_s, g->geo);
                OFDFT_LAUNCH_CHECK();
                k_pp_grad_moments<T><<<gblk, 256, 0, st>>>(rhoG, SG, nullptr, nullptr, p->line(s), g->geo, scale, mom,
                                                           mom + 4 * (size_t)nint);
            }
            OFDFT_LAUNCH_CHECK();
        }
        std::vector<double> h(4 * (size_t)nint + 3);
        OFDFT_CK(cudaMemcpyAsync(h.data(), mom, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        const int np = p->npts[s];
        double* gs = grad + off;
        for (int k = 0; k < np; ++k) gs[k] = 0.0;
        // spline over vp[1:]: d vline / d c_{l,p} = u^p, then the transpose of the fit
        std::vector<double> gc(h.begin(), h.begin() + 4 * (size_t)nint);
        std::vector<double> gy = p->spl[s].adjoint(gc);
        for (int k = 0; k < np - 1; ++k) gs[k + 1] += gy[k];
        // quartic near q = 0 in vp[0], vp[1], vp[2]
        gs[0] += h[4 * nint + 0];
        gs[1] += h[4 * nint + 1];
        gs[2] += h[4 * nint + 2];
        off += np;
    }
}

}  // namespace

extern "C" {

int ofdft_pseudo_vloc_grad(ofdft_pseudo* p, const void* rho, double* grad, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(p && rho && grad, "ofdft_pseudo_vloc_grad: null argument");
        OFDFT_REQUIRE(p->nat > 0, "ofdft_pseudo_vloc_grad: no ions set");
        if (p->g->prec == OFDFT_F64) vloc_grad_t<double>(p, (const double*)rho, grad, (cudaStream_t)s);
        else vloc_grad_t<float>(p, (const float*)rho, grad, (cudaStream_t)s);
    });
}

int ofdft_pseudo_create(ofdft_grid* g, int nspecies, const int* npts, const double* const* gp, const double* const* vp,
                        int pme, int bspline_order, ofdft_pseudo** out) {
    return guard([&] {
        OFDFT_REQUIRE(g && npts && gp && vp && out, "ofdft_pseudo_create: null argument");
        OFDFT_REQUIRE(nspecies >= 1 && nspecies <= kMaxSpecies, "ofdft_pseudo_create: 1..%d species", kMaxSpecies);
        OFDFT_REQUIRE(bspline_order >= 3 && bspline_order <= kMaxOrder, "B-spline order must be 3..%d", kMaxOrder);
        for (int d = 0; d < 3; ++d)
            OFDFT_REQUIRE(!pme || g->nr[d] >= bspline_order,
                          "PME needs at least %d grid points per axis (stencils must not wrap onto themselves)",
                          bspline_order);
        auto* p = new ofdft_pseudo();
        p->g = g;
        p->ns = nspecies;
        p->pme = pme;
        p->order = bspline_order;
        try {
            for (int s = 0; s < nspecies; ++s) {
                OFDFT_REQUIRE(npts[s] >= 6, "radial table of species %d too short", s);
                // ReadPseudo.get_vloc_interp: splrep(gp[1:], vp[1:], k=3) (pseudo/__init__.py:689-706)
                std::vector<double> x(gp[s] + 1, gp[s] + npts[s]), y(vp[s] + 1, vp[s] + npts[s]);
                CubicSpline S;
                S.fit(x, y);
                p->spl.push_back(S);
                p->gp1.push_back(gp[s][1]);
                p->gplast.push_back(gp[s][npts[s] - 1]);
                p->dp.push_back(gp[s][1] - gp[s][0]);
                p->v0.push_back(vp[s][0]);
                p->v1.push_back(vp[s][1]);
                p->v2.push_back(vp[s][2]);
                p->npts.push_back(npts[s]);
                double *dx, *dc;
                OFDFT_CK(cudaMalloc(&dx, S.x.size() * sizeof(double)));
                OFDFT_CK(cudaMalloc(&dc, S.c.size() * sizeof(double)));
                p->d_x.push_back(dx);
                p->d_c.push_back(dc);
                upload_now(dx, S.x.data(), S.x.size() * sizeof(double));
                upload_now(dc, S.c.data(), S.c.size() * sizeof(double));
            }
            bspline_tables(g, bspline_order, &p->d_bre, &p->d_bim);
            double inv[9];
            lattice_inverse(g->lattice, inv);
            OFDFT_CK(cudaMalloc(&p->d_cinv, 9 * sizeof(double)));
            upload_now(p->d_cinv, inv, 9 * sizeof(double));
        } catch (...) {
            ofdft_pseudo_destroy(p);
            throw;
        }
        *out = p;
    });
}

void ofdft_pseudo_destroy(ofdft_pseudo* p) {
    if (!p) return;
    p->sc.release_all();
    for (auto x : p->d_x) cudaFree(x);
    for (auto x : p->d_c) cudaFree(x);
    cudaFree(p->d_pos);
    cudaFree(p->d_frac);
    cudaFree(p->d_spec);
    cudaFree(p->d_sel);
    cudaFree(p->d_bre);
    cudaFree(p->d_bim);
    cudaFree(p->d_cinv);
    cudaFree(p->d_scale);
    delete p;
}

int ofdft_pseudo_set_ions(ofdft_pseudo* p, int nat, const double* pos, const int* species) {
    return guard([&] {
        OFDFT_REQUIRE(p && nat >= 1 && pos && species, "ofdft_pseudo_set_ions: bad argument");
        for (int a = 0; a < nat; ++a)
            OFDFT_REQUIRE(species[a] >= 0 && species[a] < p->ns, "atom %d has species %d outside 0..%d", a,
                          species[a], p->ns - 1);
        p->nat = nat;
        p->pos.assign(pos, pos + 3 * (size_t)nat);
        p->spec.assign(species, species + nat);
        frac_coords(p->g->lattice, nat, pos, p->frac);
        std::vector<int> sel;
        p->sel_off.assign(p->ns + 1, 0);
        for (int s = 0; s < p->ns; ++s) {
            p->sel_off[s] = (int)sel.size();
            for (int a = 0; a < nat; ++a)
                if (species[a] == s) sel.push_back(a);
        }
        p->sel_off[p->ns] = (int)sel.size();
        std::vector<double> scale(nat, -1.0);
        cudaFree(p->d_pos);
        cudaFree(p->d_frac);
        cudaFree(p->d_spec);
        cudaFree(p->d_sel);
        cudaFree(p->d_scale);
        p->d_pos = p->d_frac = p->d_scale = nullptr;
        p->d_spec = p->d_sel = nullptr;
        OFDFT_CK(cudaMalloc(&p->d_pos, 3 * (size_t)nat * sizeof(double)));
        OFDFT_CK(cudaMalloc(&p->d_frac, 3 * (size_t)nat * sizeof(double)));
        OFDFT_CK(cudaMalloc(&p->d_spec, (size_t)nat * sizeof(int)));
        OFDFT_CK(cudaMalloc(&p->d_sel, (size_t)nat * sizeof(int)));
        OFDFT_CK(cudaMalloc(&p->d_scale, (size_t)nat * sizeof(double)));
        upload_now(p->d_pos, pos, 3 * (size_t)nat * sizeof(double));
        upload_now(p->d_frac, p->frac.data(), 3 * (size_t)nat * sizeof(double));
        upload_now(p->d_spec, species, (size_t)nat * sizeof(int));
        upload_now(p->d_sel, sel.data(), (size_t)nat * sizeof(int));
        upload_now(p->d_scale, scale.data(), (size_t)nat * sizeof(double));
        p->tiles.assign(p->ns, ofdft::PmeTiles());
        if (p->pme) {
            const int nr[3] = {p->g->nr[0], p->g->nr[1], p->g->nr[2]};
            for (int s = 0; s < p->ns; ++s)
                p->tiles[s] = ofdft::pme_tiles_build(p->sc, "pme" + std::to_string(s) + "_", p->frac.data(),
                                                     sel.data() + p->sel_off[s], p->sel_off[s + 1] - p->sel_off[s],
                                                     p->order, nr, cudaStreamPerThread);
        }
    });
}

int ofdft_pseudo_vloc(ofdft_pseudo* p, void* vreal_out, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(p && vreal_out, "ofdft_pseudo_vloc: null argument");
        OFDFT_REQUIRE(p->nat > 0, "ofdft_pseudo_vloc: no ions set");
        if (p->g->prec == OFDFT_F64) vloc_t<double>(p, (double*)vreal_out, (cudaStream_t)s);
        else vloc_t<float>(p, (float*)vreal_out, (cudaStream_t)s);
    });
}

int ofdft_pseudo_stress(ofdft_pseudo* p, const void* rho, double energy, double* stress, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(p && rho && stress, "ofdft_pseudo_stress: null argument");
        OFDFT_REQUIRE(p->nat > 0, "ofdft_pseudo_stress: no ions set");
        if (p->g->prec == OFDFT_F64) stress_t<double>(p, (const double*)rho, energy, stress, (cudaStream_t)s);
        else stress_t<float>(p, (const float*)rho, energy, stress, (cudaStream_t)s);
    });
}

int ofdft_pseudo_forces(ofdft_pseudo* p, const void* rho, double* forces, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(p && rho && forces, "ofdft_pseudo_forces: null argument");
        OFDFT_REQUIRE(p->nat > 0, "ofdft_pseudo_forces: no ions set");
        if (p->g->prec == OFDFT_F64) forces_t<double>(p, (const double*)rho, forces, (cudaStream_t)s);
        else forces_t<float>(p, (const float*)rho, forces, (cudaStream_t)s);
    });
}

}  // extern "C"
