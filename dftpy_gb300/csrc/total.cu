// Total functional evaluator: fused real-space pre/post passes, fused G-space
// kernels around cuFFT, and the density-dependent (k_F-node) nonlocal kernel.
//
// One E+V evaluation (TotalFunctional.compute, src/dftpy/functional/
// total_functional.py:107-146) is:
//   pre-pass   read rho (+ v_loc): TF, LDA and PP energies and potentials,
//              sqrt(rho) for vW, rho^beta / rho^alpha and k_F for the nonlocal
//              term, float64 block partials of every energy and of
//              min/max k_F and max rho;
//   R2C        rho (Hartree), sqrt(rho) (vW), rho^beta (+ rho^alpha);
//   G-space    4 pi/G^2, G^2/2 and the Wang-Teter kernel applied in place,
//              G computed from the index (nothing stored);
//   C2R        back to real space;
//   k_F nodes  (density-dependent kernel only) batched per-node kernels, C2R,
//              interpolation, hat-weighted R2C and the pot2 accumulation;
//   post-pass  combine everything into V and the remaining energies.
#include "common.cuh"
#include "pointwise.cuh"
#include "gga.cuh"
#include "host_math.h"

#include <algorithm>
#include <type_traits>
#include <cstring>

using namespace ofdft;
using namespace ofdft::gga;

namespace {

constexpr int kMaxNodes = 4096;

template <typename T>
struct PreArgs {
    const T* rho;
    const T* vloc;
    const T* vext;  // frozen external potential (ExternalPotential)
    T* V;
    T* sq;
    T* rb;
    T* ra;
    T* kf;
    long long N;
    int tf, vw, xc, pp, ext, nl, lwt, same_ab, wantV;
    int tf_v;       // add the TF potential (off under WTE, which scales it afterwards)
    int dttf, dttf_old;
    double temp;    // DTTF temperature (Hartree) and the TF-energy x
    int nl_is_lwt;  // clamp rule: LWT clamps rho<=0, WT clamps rho<1e-30
    double tf_x;
    double alpha, beta;
    Consts k;
};

// slots: 0 TF, 1 XC, 2 PP, 3 sum rho, 4 min kF, 5 max kF, 6 max rho, 7 external, 8 DTTF
constexpr int PRE_NS = 9;

// Pointwise pre-pass.  All arithmetic runs in the grid precision T; sums run
// per thread in RunSum<T> and across threads in float64.
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_prepass(PreArgs<T> a, double* partials) {
    using M = T;
    RunSum<M> sum[6];
    M kfmin = (M)INFINITY, kfmax = -(M)INFINITY, rmax = -(M)INFINITY;
    const int kinds[PRE_NS] = {0, 0, 0, 0, 1, 2, 2, 0, 0};
    const M cTF_E = (M)a.k.cTF_E, cTF_V = (M)a.k.cTF_V, tf_x = (M)a.tf_x;
    const LdaC<M> lc(a.k);
    const M threepi2 = (M)a.k.threepi2, alpha = (M)a.alpha, beta = (M)a.beta;
    const M tiny = (M)1e-30, zero_clamp = (M)kZERO;
    const long long stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 2
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.N; i += stride) {
        const M r = a.rho[i];
        M v = (M)0;
        sum[3].add(r);
        rmax = r > rmax ? r : rmax;
        if (a.tf) {
            // PowerInt(rho, 5, 3): repeated products then cbrt (math_utils.py:158-176)
            M r5 = r * r;
            r5 *= r;
            r5 *= r;
            r5 *= r;
            sum[0].add(mcbrt(r5) * cTF_E);
            if (a.wantV && a.tf_v) v += cTF_V * mcbrt(r * r) * tf_x;
        }
        if (a.xc) {
            M ex, vx;
            lda_point(r, lc, ex, vx);
            sum[1].add(ex * r);
            v += vx;
        }
        if (a.pp) {
            const M vl = a.vloc[i];
            sum[2].add(vl * r);
            v += vl;
        }
        if (a.dttf) {  // TTF - TF (tf.py:101-204): theta = T / v_TF, fitted forms below/above 1.36
            const M T = (M)a.temp, vtf = cTF_V * mcbrt(r * r), th = T / vtf, cc = (M)0.752252778063675;
            const M r2 = sqrt((M)2), r23 = (M)2 * r2;  // 2^0.5, 2^1.5
            const M tf_ed = mcbrt(r * r * r * r * r) * cTF_E;
            const M t32 = (M)1 / sqrt(th * th * th);
            const bool hi = th >= (M)1.36;
            M vt;
            if (hi)
                vt = T * (mlog(cc * t32) + mlog((M)1 + cc * t32 / r23)) - vtf;
            else
                vt = vtf * (th * ((M)0.016 + th * ((M)-0.957 + th * ((M)-0.293 + th * (M)0.209))));
            M ed;
            if (a.dttf_old) {  // TemperatureTFEnergy_old (tf.py:180-204)
                const M th52 = sqrt(th * th * th * th * th);
                ed = (vt + vtf) * r - (M)(2.0 * 1.4142135623730951 / 3.0 / (M_PI * M_PI)) * (T * T * sqrt(T)) / th52 *
                                         sqrt((M)0.16 + th * th) /
                                         ((M)1 - (M)0.14 * (mexp(-th) - mexp((M)-3.68 * th))) -
                     tf_ed;
            } else if (hi) {  // TemperatureTFEnergy (tf.py:134-177)
                const M k = T / cTF_V;
                ed = ((M)-2 * r + r23 * k * sqrt(k) * atanh(cc * t32 / r23) / cc + r * mlog((M)1 + cc / r23 * t32) +
                      r * mlog(cc * t32) + r2 * k * sqrt(th) * mcbrt(r) * mlog((M)8 * k * k * k - cc * cc * (r * r)) / cc) *
                         T -
                     tf_ed;
            } else {
                ed = T * (r * ((M)0.016 + th * ((M)(-0.957 * 3) + th * ((M)(-0.293 * -3) + th * (M)-0.209))));
            }
            sum[5].add(ed);
            if (a.wantV) v += vt * tf_x;
        }
        if (a.ext) {  // external_potential.py:30-35
            const M ve = a.vext[i];
            sum[4].add(ve * r);
            v += ve;
        }
        if (a.vw) a.sq[i] = msqrt(r > (M)0 ? r : tiny);  // kedf/vw.py:34-44
        if (a.nl) {
            const M rc = a.nl_is_lwt ? (r > (M)0 ? r : tiny) : (r < zero_clamp ? zero_clamp : r);
            a.rb[i] = mpow(rc, beta);
            if (!a.same_ab) a.ra[i] = mpow(rc, alpha);
        }
        if (a.lwt) {
            const M kf = (M)2 * mcbrt(threepi2 * r);  // kedf/lwt.py:106
            a.kf[i] = kf;
            kfmin = kf < kfmin ? kf : kfmin;
            kfmax = kf > kfmax ? kf : kfmax;
        }
        if (a.wantV) a.V[i] = v;
    }
    double acc[PRE_NS] = {sum[0].get(), sum[1].get(), sum[2].get(), sum[3].get(), (double)kfmin, (double)kfmax,
                          (double)rmax, sum[4].get(), sum[5].get()};
    block_reduce_store<PRE_NS>(acc, kinds, partials);
}

// --------------------------------------------------------------- G space
template <typename T>
struct GArgs {
    typename Cplx<T>::type* rhoG;  // in: FFT(rho)  out: v_H(G)/N
    typename Cplx<T>::type* sqG;   // in: FFT(sqrt rho) out: G^2/2 FFT / N
    typename Cplx<T>::type* rbG;   // in: FFT(rho^beta) out: K FFT / N (WT)
    typename Cplx<T>::type* raG;   // in: FFT(rho^alpha) out: K FFT / N (WT, alpha != beta)
    T* wtK;                        // cached WT kernel (Nc)
    const double* wtstate;         // [saved rho0, recompute flag, tkf, factor]
    double wt_x;
    double vw_s;                   // sigma^2/4 of the vW smoothing (0: none)
    int mgp;                       // the kernel comes from k_mgp_kernel
    Geo geo;
    double invN;
};

template <typename T>
__global__ void k_gspace(GArgs<T> a) {
    using M = T;  // working precision of the multipliers
    const long long stride = (long long)gridDim.x * blockDim.x;
    const bool recompute = a.wtK && a.wtstate[1] != 0.0 && !a.mgp;
    const M invN = (M)a.invN, fourpi = (M)(4.0 * M_PI), half = (M)0.5;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.geo.Nc; i += stride) {
        const M gg = gsq_t<M>(a.geo, i);
        if (a.rhoG) {  // Hartree: 4 pi / G^2, G=0 -> 0 (hartree.py:33-35, grid.py:532-541)
            const M f = (i == 0) ? (M)0 : fourpi / gg * invN;
            auto z = a.rhoG[i];
            z.x = z.x * f;
            z.y = z.y * f;
            a.rhoG[i] = z;
        }
        if (a.sqG) {  // vW: G^2 (vw.py:45-51) with the 1/2 folded in, smoothed with sigma (:47-48)
            M f = half * gg * invN;
            if (a.vw_s > 0.0) f *= mexp(-gg * (M)a.vw_s);
            auto z = a.sqG[i];
            z.x = z.x * f;
            z.y = z.y * f;
            a.sqG[i] = z;
        }
        if (a.wtK) {  // Wang-Teter kernel (kernel.py:325-334), cached per rho0, built in float64
            M K;
            if (recompute) {
                const double q = sqrt(gsq(a.geo, i));
                K = (M)(lindhard_dev(q / a.wtstate[2], a.wt_x, 1.0) * a.wtstate[3]);
                a.wtK[i] = K;
            } else {
                K = a.wtK[i];
            }
            const M f = K * invN;
            auto z = a.rbG[i];
            z.x = z.x * f;
            z.y = z.y * f;
            a.rbG[i] = z;
            if (a.raG) {
                auto w = a.raG[i];
                w.x = w.x * f;
                w.y = w.y * f;
                a.raG[i] = w;
            }
        }
    }
}

// device-side WT kernel cache decision (wt.py:58-73): rebuild when rho0 moves by > 1e-6
__global__ void k_wt_plan(const double* results, double* state, double rho0_fixed, double invN, double alpha,
                          double beta, double cTF) {
    double rho0 = rho0_fixed > 0.0 ? rho0_fixed : results[3] * invN;
    bool first = state[4] == 0.0;
    if (first || fabs(state[0] - rho0) > 1e-6) {
        state[0] = rho0;
        state[1] = 1.0;
        state[2] = 2.0 * pow(3.0 * rho0 * (M_PI * M_PI), 1.0 / 3.0);
        state[3] = 5.0 / (9.0 * alpha * beta * pow(rho0, alpha + beta - 5.0 / 3.0)) * cTF;
        state[4] = 1.0;
    } else {
        state[1] = 0.0;
    }
}

// ------------------------------------------------------------ MGP kernels
struct MgpArgs {
    const double* x;  // spline data points (log-spaced eta)
    const double* c;  // 4 per interval
    int n;
    int maxpoints, sym, lump, revke;
    double abc[3];
    double volume;
};

// splev(eta, table, ext=3) of the Lindhard spline: the boundary value outside the table
__device__ inline double mgp_splev(const MgpArgs& m, double v) {
    if (v <= m.x[0]) return m.c[0];
    if (v >= m.x[m.n - 1]) {
        const double* p = m.c + 4 * (m.n - 2);
        const double u = m.x[m.n - 1] - m.x[m.n - 2];
        return p[0] + u * (p[1] + u * (p[2] + u * p[3]));
    }
    int lo = 0, hi = m.n - 1;  // x[lo] <= v < x[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (m.x[mid] <= v)
            lo = mid;
        else
            hi = mid;
    }
    const double* p = m.c + 4 * lo;
    const double u = v - m.x[lo];
    return p[0] + u * (p[1] + u * (p[2] + u * p[3]));
}

// MGPKernel + MGPOmegaE at the saved rho0 (mgp.py:39-46, kernel.py:251-322, 408-440),
// written when k_wt_plan flagged a rebuild (state[1]); K(G=0) = 0.
template <typename T>
__global__ void k_mgp_kernel(T* K, Geo geo, const double* state, MgpArgs m) {
    if (state[1] == 0.0) return;
    const double rho0 = state[0], tkf = state[2];
    const double cTF = 0.3 * pow(3.0 * M_PI * M_PI, 2.0 / 3.0), dt = 1.0 / m.maxpoints;
    const double coe = 4.0 / 5.0 * cTF * 5.0 / 6.0 * dt;
    double a = m.abc[0], b = m.abc[1];
    if (m.lump == 1) {
        a = a / pow(rho0 * m.volume, 2.0 / 3.0);
        b = a;
    }
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < geo.Nc; idx += stride) {
        if (idx == 0) {
            K[0] = (T)0;
            continue;
        }
        const double q = sqrt(gsq(geo, idx));
        const double eta = q / tkf;
        double s = 0.0;
        for (int i = 1; i <= m.maxpoints; ++i) {
            const double t = i * dt;
            const double t16 = m.sym == 2 ? pow(t, -2.0 / 3.0) : pow(t, 1.0 / 6.0);
            s += mgp_splev(m, eta / cbrt(t)) / t16;
        }
        double k;
        if (m.sym == 1)
            k = 0.5 * (s * coe + lindhard_dev(eta, 1.0, 1.0) * (4.0 / 5.0 * cTF));
        else if (m.sym == 2)
            k = s * (2.0 * coe);
        else
            k = s * coe;
        if (m.lump) {
            const double gg = q * q;
            const double er = m.revke ? erf(m.abc[2] * gg) : erf(m.abc[2] * q);
            double corr = 4.0 * M_PI * er * er * a * exp(-gg * b) / gg;
            if (!m.revke) corr *= 3.0 / 5.0;
            k += corr;
        }
        K[idx] = (T)k;
    }
}

// ----------------------------------------------------- density-dependent kernel
// Kernel table K(eta) and derivative table -eta K'(eta) as cubic pieces on the
// uniform eta grid of the reference (lwt.py:535-566).
template <typename T>
struct Table {
    const T* c;      // 4 per interval
    const T* cd;     // derivative table
    int nint;        // neta - 1
    double step, inv_step, etamax;
    double limit, limitd;  // values at etamax
    double factor, lbda;   // table = factor * F(eta; lbda, 1); closed form used above eta_series
    double eta_series;     // FP32 path: closed-form large-eta series at and above this eta
    int hc;                // HC scaling (HCKernelXi, kernel.py:496-506): node inverses are 1/(2k)
};

// Node kernel and derivative kernel of one node from the table values K, KD at
// eta = q c: LWT K and KD c (c = 1/k); HC (c = 1/(2k)) K c^3 and (KD - 3K) c^3 2c.
template <typename T>
__device__ inline void scale_node(const Table<T>& tab, T c, T& K, T& kd, T KD) {
    if (tab.hc) {
        const T c3 = c * c * c;
        kd = (KD - (T)3 * K) * c3 * ((T)2 * c);
        K = K * c3;
    } else {
        kd = KD * c;
    }
}

// Large-eta branch of the inverse Lindhard function (kernel.py:79-133) with
// mu = 1: F = -lbda - 0.6 + sum_k c_k eta^{-2k}, and -eta dF/deta = sum_k 2k c_k
// eta^{-2k}.  The series converges for eta > 1; the reference's table holds it
// above eta = 3.65 (kernel.py:27) and the same function in closed form below, so
// at and above eta = 2.5 the truncated series reproduces the table to ~5e-10 of F
// (below float32 resolution) and the FP32 paths evaluate it in registers there.
__constant__ float cLargeF[15] = {-0.13714285714285712f, -6.39999999999999875e-2f, -3.77825602968460128e-2f,
                                  -2.51824061652633074e-2f, -1.80879839616166146e-2f, -1.36715733124818332e-2f,
                                  -1.07236045520990083e-2f, -8.65192783339199453e-3f, -7.1372762502456763e-3f,
                                  -5.9945117538835746e-3f, -5.10997527675418131e-3f, -4.41060829979912465e-3f,
                                  -3.84763737842981233e-3f, -3.38745061493813488e-3f, -3.00624946457977689e-3f};

__device__ inline void large_eta_series(float eta, float factor, float lbda, bool deriv, float& K, float& KD) {
    const float inv2 = 1.0f / (eta * eta);
    float f = cLargeF[14], d = 30.0f * cLargeF[14];
#pragma unroll
    for (int k = 13; k >= 0; --k) {
        f = fmaf(f, inv2, cLargeF[k]);
        if (deriv) d = fmaf(d, inv2, (float)(2 * (k + 1)) * cLargeF[k]);
    }
    K = factor * (-lbda - 0.6f + f * inv2);
    KD = deriv ? factor * d * inv2 : 0.0f;
}

// one interval's four coefficients in a single vector load (rows are 16 B
// aligned for float32, 32 B for float64; the table is read through L2)
__device__ inline float4 coef4(const float* c, int l) { return __ldg(reinterpret_cast<const float4*>(c) + l); }
__device__ inline double4 coef4(const double* c, int l) {
    const double2* p = reinterpret_cast<const double2*>(c) + 2 * (long long)l;
    double2 a = __ldg(p), b = __ldg(p + 1);
    return make_double4(a.x, a.y, b.x, b.y);
}

template <typename T>
__device__ inline T spline_eval(const T* c, int nint, T step, T inv_step, T eta) {
    int l = (int)(eta * inv_step);
    l = l < 0 ? 0 : (l >= nint ? nint - 1 : l);
    T u = eta - (T)l * step;
    const auto q = coef4(c, l);
    return q.x + u * (q.y + u * (q.z + u * q.w));
}

struct Nodes {
    const double* k;     // node k_F
    const double* invk;  // 1/k
};

// Node kernel values in the working precision T: K_j(|G|) for eta = |G|/k_j
// below etamax (spline), the etamax value above it, 0 at G = 0.
template <typename T>
__device__ inline void node_kernel(const Table<T>& tab, T q, T invk, bool deriv, long long i, T& K, T& KD) {
    const T eta = q * invk;
    KD = (T)0;
    if (eta < (T)tab.etamax) {
        if (sizeof(T) == 4 && eta >= (T)tab.eta_series) {
            float k, kd;
            large_eta_series((float)eta, (float)tab.factor, (float)tab.lbda, deriv, k, kd);
            K = (T)k;
            KD = (T)kd;
        } else {
            K = spline_eval(tab.c, tab.nint, (T)tab.step, (T)tab.inv_step, eta);
            if (deriv) KD = spline_eval(tab.cd, tab.nint, (T)tab.step, (T)tab.inv_step, eta);
        }
    } else {
        K = (T)tab.limit;
        KD = (T)tab.limitd;
    }
    if (i == 0) K = KD = (T)0;
}

// X_j = K_j(G) FFT(rho^beta)/N and Y_j = K'_j(G)/k_j FFT(rho^beta)/N for the
// chunk's nodes (LWTKernelKf, kernel.py:379-405; lwt.py:226-251).  The node
// reciprocals of the chunk sit in shared memory.
template <typename T>
__global__ void k_lwt_nodes(const typename Cplx<T>::type* __restrict__ rbG, typename Cplx<T>::type* __restrict__ XY,
                            Table<T> tab, Nodes nd, int j0, int nb, int mcalc, Geo geo, double invN) {
    extern __shared__ unsigned char smem_nodes[];
    T* sinvk = (T*)smem_nodes;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) sinvk[t] = (T)nd.invk[j0 + t];
    __syncthreads();
    const T invNt = (T)invN;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        const T q = sqrt(gsq_t<T>(geo, i));
        const auto z = rbG[i];
        const T zr = z.x * invNt, zi = z.y * invNt;
        for (int jj = 0; jj < nb; ++jj) {
            T K, KD, kd;
            node_kernel(tab, q, sinvk[jj], mcalc != 0, i, K, KD);
            scale_node(tab, sinvk[jj], K, kd, KD);
            typename Cplx<T>::type o;
            o.x = K * zr;
            o.y = K * zi;
            XY[(long long)jj * geo.Nc + i] = o;
            if (mcalc) {
                o.x = kd * zr;
                o.y = kd * zi;
                XY[(long long)(nb + jj) * geo.Nc + i] = o;
            }
        }
    }
}

// pot2G (+)= sum_j K_j(G) U_j(G)/N [+ K'_j/k_j UD_j(G)/N] (lwt.py:266-296)
template <typename T>
__global__ void k_lwt_pot2(const typename Cplx<T>::type* __restrict__ U, typename Cplx<T>::type* __restrict__ pot2G,
                           Table<T> tab, Nodes nd, int j0, int nb, int hermite, int first, Geo geo, double invN) {
    extern __shared__ unsigned char smem_nodes[];
    T* sinvk = (T*)smem_nodes;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) sinvk[t] = (T)nd.invk[j0 + t];
    __syncthreads();
    const T invNt = (T)invN;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        const T q = sqrt(gsq_t<T>(geo, i));
        T sr = 0, si = 0;
        if (!first) {
            sr = pot2G[i].x;
            si = pot2G[i].y;
        }
        for (int jj = 0; jj < nb; ++jj) {
            T K, KD, kd0;
            node_kernel(tab, q, sinvk[jj], hermite != 0, i, K, KD);
            scale_node(tab, sinvk[jj], K, kd0, KD);
            const auto u = U[(long long)jj * geo.Nc + i];
            sr += K * invNt * u.x;
            si += K * invNt * u.y;
            if (hermite) {
                const T kd = kd0 * invNt;
                const auto w = U[(long long)(nb + jj) * geo.Nc + i];
                sr += kd * w.x;
                si += kd * w.y;
            }
        }
        typename Cplx<T>::type o;
        o.x = sr;
        o.y = si;
        pot2G[i] = o;
    }
}

// per-point interval membership of the reference (lwt.py:252-306):
// interval i holds kf in (k_i, k_{i+1} + 1e-18); 'small' holds kf < k_0 + 1e-18.
struct Member {
    int ilast, iprev;  // last / previous containing interval, -1 if none
    bool small;
};

// closed_interior: a point exactly on an interior node joins the interval below
// it.  Float32 k_F values tie with interior nodes now and then (the nodes are
// built from float32 extremes); the open test of the reference would then drop
// the point from every interval.  Float64 keeps the reference's test exactly.
__device__ inline Member membership(double kf, const double* kn, const double* kup, int m, bool closed_interior) {
    // c = number of nodes strictly below kf
    int lo = 0, hi = m;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (kn[mid] < kf) lo = mid + 1;
        else hi = mid;
    }
    const int c = lo;
    Member r;
    r.ilast = -1;
    r.iprev = -1;
    int i1 = c - 1, i2 = c - 2;
    auto below_top = [&](int i) {
        return (closed_interior && i + 1 <= m - 2) ? kf <= kn[i + 1] : kf < kup[i + 1];
    };
    bool in1 = (i1 >= 0 && i1 <= m - 2 && below_top(i1));
    bool in2 = (i2 >= 0 && i2 <= m - 2 && below_top(i2));
    if (in1) {
        r.ilast = i1;
        if (in2) r.iprev = i2;
    } else if (in2) {
        r.ilast = i2;
    }
    r.small = kf < kup[0];
    return r;
}

template <typename T>
struct InterpArgs {
    const T* kf;
    const T* rA;
    const T* PM;  // P planes then M planes of the chunk
    T* pot1;
    T* pot3;
    T* u;         // nb (linear) or 2 nb (hermite) planes
    const double* kn;
    const double* kup;  // k_i + 1e-18
    int m, j0, nb, kdd, hermite, mcalc, first;
    double kfclip;
    long long N;
};

template <typename T>
__global__ void k_lwt_interp(InterpArgs<T> a) {
    using M = T;  // working precision of the weights; membership tests stay float64
    extern __shared__ double sh[];
    double* kn = sh;
    double* kup = sh + a.m;
    for (int t = threadIdx.x; t < a.m; t += blockDim.x) {
        kn[t] = a.kn[t];
        kup[t] = a.kup[t];
    }
    __syncthreads();
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int j1 = a.j0 + a.nb;
    // interval coordinate t = (kf - k_i) / (k_{i+1} - k_i), as the reference divides
    auto tcoord = [&](double kf, int i) { return (M)(kf - kn[i]) / (M)(kn[i + 1] - kn[i]); };
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < a.N; r += stride) {
        const double kf = fmin((double)a.kf[r], a.kfclip);
        const Member mb = membership(kf, kn, kup, a.m, sizeof(T) == 4);
        M p1 = (M)0, p3 = (M)0;
        auto P = [&](int j) { return a.PM[(long long)(j - a.j0) * a.N + r]; };
        auto Md = [&](int j) { return a.PM[(long long)(a.nb + j - a.j0) * a.N + r]; };
        if (mb.ilast >= 0) {
            const int i = mb.ilast;
            const M D = (M)(kn[i + 1] - kn[i]);
            const M t = tcoord(kf, i);
            if (!a.hermite) {
                const M t0 = (M)1 - t;
                if (i >= a.j0 && i < j1) {
                    p1 += P(i) * t0;
                    if (a.kdd == 3) p3 += Md(i) * t0;
                }
                if (i + 1 >= a.j0 && i + 1 < j1) {
                    p1 += P(i + 1) * t;
                    if (a.kdd == 3) p3 += Md(i + 1) * t;
                }
            } else {
                const M t2 = t * t, t3 = t2 * t;
                const M h00 = (M)2 * t3 - (M)3 * t2 + (M)1, h10 = t3 - (M)2 * t2 + t, h01 = (M)1 - h00,
                        h11 = t3 - t2;
                const M h00D = (M)6 * t2 - 6 * t, h10D = (M)3 * t2 - 4 * t + (M)1, h01D = -h00D,
                        h11D = (M)3 * t2 - 2 * t;
                if (i >= a.j0 && i < j1) {
                    p1 += h00 * P(i) + D * h10 * Md(i);
                    if (a.kdd == 3) p3 += h00D * P(i) / D + h10D * Md(i);
                }
                if (i + 1 >= a.j0 && i + 1 < j1) {
                    p1 += h01 * P(i + 1) + D * h11 * Md(i + 1);
                    if (a.kdd == 3) p3 += h01D * P(i + 1) / D + h11D * Md(i + 1);
                }
            }
        } else if (mb.small) {
            const M ts = (M)(kf - kn[0]) / (M)kn[0];
            if (a.j0 == 0) p1 += P(0) * ts;
        }
        if (a.first) {
            a.pot1[r] = p1;
            if (a.kdd == 3) a.pot3[r] = p3;
        } else {
            a.pot1[r] = a.pot1[r] + p1;
            if (a.kdd == 3) a.pot3[r] = a.pot3[r] + p3;
        }
        if (a.kdd > 1) {
            // hat weights W_j (and WD_j for hermite) of every containing interval;
            // at most three distinct nodes: base, base+1, base+2
            const M rA = a.rA[r];
            const int ints[2] = {mb.ilast, mb.iprev};
            const int base = mb.ilast >= 0 ? (mb.iprev >= 0 ? mb.iprev : mb.ilast) : 0;
            M W[3] = {0, 0, 0}, WD[3] = {0, 0, 0};
            for (int q = 0; q < 2; ++q) {
                const int i = ints[q];
                if (i < 0) continue;
                const M t = tcoord(kf, i);
                if (!a.hermite) {
                    W[i - base] += (M)1 - t;
                    W[i + 1 - base] += t;
                } else {
                    const M D = (M)(kn[i + 1] - kn[i]);
                    const M t2 = t * t, t3 = t2 * t;
                    const M h00 = (M)2 * t3 - (M)3 * t2 + (M)1, h10 = t3 - (M)2 * t2 + t, h01 = (M)1 - h00,
                            h11 = t3 - t2;
                    W[i - base] += h00;
                    W[i + 1 - base] += h01;
                    WD[i - base] += D * h10;
                    WD[i + 1 - base] += D * h11;
                }
            }
            const M ws0 = mb.small ? (M)(kf - kn[0]) / (M)kn[0] : (M)0;
            for (int jj = 0; jj < a.nb; ++jj) {
                const int j = a.j0 + jj;
                M wj = (M)0, wdj = (M)0;
                const int d = j - base;
                if (mb.ilast >= 0 && d >= 0 && d < 3) {
                    wj = W[d];
                    wdj = WD[d];
                }
                if (j == 0) wj += ws0;
                a.u[(long long)jj * a.N + r] = rA * wj;
                if (a.hermite) a.u[(long long)(a.nb + jj) * a.N + r] = rA * wdj;
            }
        }
    }
}

// ------------------------------------------------------------- post-pass
template <typename T>
struct PostArgs {
    const T* rho;
    T* V;
    T* Vnl;  // WTE: the WT potential goes here instead of into V
    const T* sq;
    const T* lap;   // (1/2) IFFT(G^2 FFT(sqrt rho)) (already normalised)
    const T* vH;
    const T* nl1;   // IFFT(K FFT(rho^beta))
    const T* nl2;   // IFFT(K FFT(rho^alpha)) (alpha != beta)
    const T* rb;
    const T* ra;
    // LWT
    const T* kf;
    const T* pot1;
    const T* pot2;
    const T* pot3;
    // HC: c1 = k_F,std (F - 4 F' s^2)/(3 rho) and the divergence term
    int hc;
    const T* hc_c1;
    const T* hc_q;
    long long N;
    int vw, h, wt, lwt, same_ab, wantV, kdd;
    double vw_y;
    double alpha, beta;  // of the active nonlocal term
    double rhomax, ld, kfclip;
};

// slots: 0 vW, 1 Hartree, 2 NL
constexpr int POST_NS = 3;

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_postpass(PostArgs<T> a, double* partials) {
    using M = T;  // working precision; sums run in RunSum<T>, then float64
    RunSum<M> sum[POST_NS];
    const M alpha = (M)a.alpha, beta = (M)a.beta, vw_y = (M)a.vw_y, ld = (M)a.ld, rhomax = (M)a.rhomax;
    const M kfclip = (M)a.kfclip, tiny = (M)1e-30, zero_clamp = (M)kZERO;
    const long long stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 2
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.N; i += stride) {
        const M r = a.rho[i];
        M v = a.wantV ? a.V[i] : (M)0;
        if (a.vw) {
            M s = a.sq[i];
            if (fabs(s) < tiny) s = tiny;
            const M pw = a.lap[i] / s;
            if (r > (M)0) sum[0].add(r * pw);
            v += pw * vw_y;
        }
        if (a.h) {
            const M vh = a.vH[i];
            sum[1].add(vh * r);
            v += vh;
        }
        if (a.wt) {
            const M rc = r < zero_clamp ? zero_clamp : r;
            const M pb = a.rb[i];
            const M c1 = a.nl1[i];
            M vnl = (M)0;
            if (a.same_ab) {
                const M pot = (M)2 * alpha * (pb / rc) * c1;  // wt.py:19-23
                if (a.wantV) {
                    sum[2].add(pot * r / ((M)2 * alpha));  // wt.py:124-125
                    vnl = pot;
                } else {
                    sum[2].add(c1 * pb);  // wt.py:44-56
                }
            } else {
                const M pa = a.ra[i];
                sum[2].add(c1 * pa);
                if (a.wantV) vnl = alpha * (pa / rc) * c1 + beta * (pb / rc) * a.nl2[i];
            }
            if (a.wantV) {
                if (a.Vnl)
                    a.Vnl[i] = vnl;
                else
                    v += vnl;
            }
        }
        if (a.lwt && a.hc) {
            // HC (hc.py:294-330): the energy without the low-density factor, the potential
            // factor * (alpha rho^(alpha-1) pot1 + beta rho^(beta-1) pot2 + c1 rho^alpha pot3 - div)
            const M rc = r < zero_clamp ? zero_clamp : r;
            const M pa = a.same_ab ? a.rb[i] : a.ra[i];
            sum[2].add(pa * a.pot1[i]);
            if (a.wantV) {
                M f = (M)1;
                if (rc < (M)1e-6) f = mpow(fabs(rc), ld) / mpow(rhomax, ld);
                const M pb = a.rb[i];
                v += f * (alpha * (pa / rc) * a.pot1[i] + beta * (pb / rc) * a.pot2[i] + a.hc_c1[i] * pa * a.pot3[i] -
                          a.hc_q[i]);
            }
        } else if (a.lwt) {
            // low-density factor (lwt.py:315-322) and the final combination (:324-339)
            M f = (M)1;
            if (r < (M)1e-6) f = mpow(fabs(r), ld) / mpow(rhomax, ld);
            if (r < (M)0) f = (M)0;
            const M rc = r > (M)0 ? r : tiny;
            const M pa = a.same_ab ? a.rb[i] : a.ra[i];
            const M p1 = a.pot1[i] * f;
            sum[2].add(pa * p1);
            if (a.wantV) {
                const M pb = a.rb[i];
                const M p2 = (a.kdd > 1 ? a.pot2[i] : a.pot1[i]) * f;
                const M p3 = (a.kdd == 3 ? a.pot3[i] : (M)0) * f;
                const M kfv = a.kf[i];
                const M kf = kfv < kfclip ? kfv : kfclip;
                v += alpha * (pa / rc) * p1 + (beta * (pb / rc) * p2 + (kf / (M)3) * (pa / rc) * p3);
            }
        }
        if (a.wantV) a.V[i] = v;
    }
    double acc[POST_NS] = {sum[0].get(), sum[1].get(), sum[2].get()};
    block_sum_store<POST_NS>(acc, partials);
}

// WTE potential (wte.py:15-18) from the prepass TF sum (R0[0]) and the
// postpass WT sum (R16[2]): V += exp(r) ((1 - r) V_TF + V_WT), r = E_WT / E_TF.
template <typename T>
__global__ void k_wte_combine(const T* __restrict__ rho, T* V, const T* __restrict__ Vnl, long long N,
                              const double* R0, const double* R16, double dV, double tf_x, double cTF_V) {
    const double etf = R0[0] * dV * tf_x, ewt = R16[2] * dV;
    const double r = ewt / etf, ex = exp(r);
    const T c1 = (T)(ex * (1.0 - r)), c2 = (T)ex, ctf = (T)cTF_V, tx = (T)tf_x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const T x = rho[i];
        V[i] += c1 * (ctf * mcbrt(x * x) * tx) + c2 * Vnl[i];
    }
}

template <typename T>
__global__ void k_zero(T* p, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = (T)0;
}

}  // namespace

#include "lwt_split.cuh"

// ------------------------------------------------------------------ handle
struct ofdft_eval {
    ofdft_grid* g = nullptr;
    ofdft_config cfg;
    Consts k;
    Scratch sc;
    void* vloc = nullptr;  // grid precision
    bool have_vloc = false;
    void* vext = nullptr;  // grid precision
    bool have_vext = false;
    // MGP kernels of the WT term: the Lindhard spline on the log-spaced eta table
    double* mgp_x = nullptr;  // knots (data points)
    double* mgp_c = nullptr;  // 4 per interval
    int mgp_n = 0;
    bool tab_set = false;  // the k_F-node kernel table is on the device
    double* wtstate = nullptr;  // device [rho0, flag, tkf, factor, init]
    // density-dependent kernel
    void* tab_c = nullptr;
    void* tab_cd = nullptr;
    int tab_nint = 0;
    double tab_step = 0, tab_limit = 0, tab_limitd = 0;
    double* d_nodes = nullptr;  // [k (kMaxNodes), 1/k, k+1e-18]
    double* h_nodes = nullptr;  // pinned staging
    float2* fz_tw = nullptr;    // twiddle tables of the fused k_F-node pipeline
    unsigned* d_fz_err = nullptr;  // fused pipeline: nonzero after a bulk copy that did not complete
    cudaStream_t fz_st2 = nullptr;     // fused pipeline: the R2C chain runs here, beside the C2R chain
    cudaEvent_t fz_fork = nullptr, fz_join = nullptr;
    unsigned* h_fz_err = nullptr;  // pinned mirror
    bool fz_ran = false;           // the last evaluation ran the fused pipeline
    // terms of an evaluation whose energies have not been collected yet
    struct Pending {
        bool tf, vw, wt, lwt, xc, h, pp, ext, lp_active, gga;
        int launches;
    } pend{};
    bool kf_set_min = false, kf_set_max = false;
    double kf_st_min = 0, kf_st_max = 0;
    int last_nsp = 0, last_launches = 0;
    // per-kernel-class CUDA-event profiling
    static constexpr int kClasses = 10;
    bool prof = false;
    std::vector<cudaEvent_t> evs;   // pool, two per recorded launch
    std::vector<int> rec_cls;       // class of each recorded launch
    std::vector<double> rec_bytes;  // algorithmic bytes of each recorded launch
    double prof_ms[kClasses] = {0};
    double prof_bytes[kClasses] = {0};
    long long prof_launches[kClasses] = {0};
};

ofdft_grid* e_grid(ofdft_eval* e) { return e->g; }
const ofdft_config* e_cfg(const ofdft_eval* e) { return &e->cfg; }
const void* e_vloc(const ofdft_eval* e) { return e->have_vloc ? e->vloc : nullptr; }

namespace {
template <typename T>
void compute_t(ofdft_eval* e, const T* rho, T* V, unsigned calc, double* energies, cudaStream_t st);
void collect_energies(ofdft_eval* e, double* energies);
}  // namespace

// For the batched optimiser: enqueue an evaluation without waiting, and read its
// energies once the stream has been synchronised.
void eval_enqueue(ofdft_eval* e, const void* rho, void* v_out, unsigned calc, cudaStream_t st) {
    if (e->g->prec == OFDFT_F64) compute_t<double>(e, (const double*)rho, (double*)v_out, calc, nullptr, st);
    else compute_t<float>(e, (const float*)rho, (float*)v_out, calc, nullptr, st);
}
void eval_collect(ofdft_eval* e, double* energies) { collect_energies(e, energies); }
// an evaluation that waits on the host mid-way (the k_F-node kernel reads its
// k_F bounds back) cannot be captured into a CUDA graph
bool eval_capturable(const ofdft_eval* e) { return !(e->cfg.kedf_terms & OFDFT_KE_LWT); }

namespace {

enum ProfClass {
    P_PREPASS = 0,
    P_GSPACE,
    P_LWT_NODES,
    P_LWT_INTERP,
    P_LWT_POT2,
    P_POSTPASS,
    P_REDUCE,
    P_CUFFT,
    P_FZ_AXIS1,
    P_FZ_HAT
};
const char* kProfNames[ofdft_eval::kClasses] = {"prepass", "gspace",   "lwt_nodes", "lwt_interp", "lwt_pot2",
                                                 "postpass", "reduce", "cufft",     "fz_axis1",   "fz_hat"};

// Record a start event for one launch of class cls moving `bytes` algorithmic bytes.
int prof_begin(ofdft_eval* e, int cls, double bytes, cudaStream_t st) {
    if (!e->prof) return -1;
    const int idx = (int)e->rec_cls.size();
    while ((int)e->evs.size() < 2 * (idx + 1)) {
        cudaEvent_t ev;
        OFDFT_CK(cudaEventCreate(&ev));
        e->evs.push_back(ev);
    }
    e->rec_cls.push_back(cls);
    e->rec_bytes.push_back(bytes);
    OFDFT_CK(cudaEventRecord(e->evs[2 * idx], st));
    return idx;
}

void prof_end(ofdft_eval* e, int idx, cudaStream_t st) {
    if (idx < 0) return;
    OFDFT_CK(cudaEventRecord(e->evs[2 * idx + 1], st));
}

// after the stream has been synchronised: fold recorded launches into the totals
void prof_collect(ofdft_eval* e) {
    for (size_t i = 0; i < e->rec_cls.size(); ++i) {
        float ms = 0.f;
        OFDFT_CK(cudaEventElapsedTime(&ms, e->evs[2 * i], e->evs[2 * i + 1]));
        e->prof_ms[e->rec_cls[i]] += ms;
        e->prof_bytes[e->rec_cls[i]] += e->rec_bytes[i];
        e->prof_launches[e->rec_cls[i]] += 1;
    }
    e->rec_cls.clear();
    e->rec_bytes.clear();
}

// run `f` (one launch) between profiling events
template <class F>
void timed(ofdft_eval* e, int cls, double bytes, cudaStream_t st, F&& f) {
    int idx = prof_begin(e, cls, bytes, st);
    f();
    prof_end(e, idx, st);
}

// splines of the table values y(eta) and of -eta y'(eta) (lwt.py:554-556), uploaded
template <typename T>
void upload_table(ofdft_eval* e, const std::vector<double>& eta, const std::vector<double>& y) {
    const int neta = (int)eta.size();
    CubicSpline S;
    S.fit(eta, y);
    std::vector<double> yd(neta);
    for (int i = 0; i < neta; ++i) yd[i] = S.deriv(eta[i]) * (-1.0 * eta[i]);  // lwt.py:556
    CubicSpline SD;
    SD.fit(eta, yd);
    const int nint = neta - 1;
    std::vector<T> hc(4 * (size_t)nint), hcd(4 * (size_t)nint);
    for (size_t i = 0; i < hc.size(); ++i) {
        hc[i] = (T)S.c[i];
        hcd[i] = (T)SD.c[i];
    }
    if (!e->tab_c) OFDFT_CK(cudaMalloc(&e->tab_c, hc.size() * sizeof(T)));
    if (!e->tab_cd) OFDFT_CK(cudaMalloc(&e->tab_cd, hcd.size() * sizeof(T)));
    upload_now(e->tab_c, hc.data(), hc.size() * sizeof(T));
    upload_now(e->tab_cd, hcd.data(), hcd.size() * sizeof(T));
    e->tab_nint = nint;
    e->tab_step = eta[1] - eta[0];
    e->tab_limit = S.eval(eta[neta - 1]);
    e->tab_limitd = SD.eval(eta[neta - 1]);
    e->tab_set = true;
}

// numpy linspace(0, etamax, neta)
std::vector<double> table_eta(const ofdft_config& c) {
    const int neta = c.lwt_neta;
    std::vector<double> eta(neta);
    const double step = c.lwt_etamax / (double)(neta - 1);
    for (int i = 0; i < neta; ++i) eta[i] = (double)i * step;
    eta[neta - 1] = c.lwt_etamax;
    return eta;
}

template <typename T>
void build_table(ofdft_eval* e) {
    const ofdft_config& c = e->cfg;
    if (c.lwt_kernel == OFDFT_LWT_KERNEL_USER) return;  // ofdft_eval_set_lwt_table supplies it
    const int neta = c.lwt_neta;
    const std::vector<double> eta = table_eta(c);
    std::vector<double> y(neta);
    if (c.lwt_kernel == OFDFT_LWT_KERNEL_WT) {
        // WTKernelTable (kernel.py:344-352): F(eta; x, 1) * (4/5) * 0.3 (3 pi^2)^(2/3)
        const double factor = 4.0 / 5.0 * 0.3 * std::pow(3.0 * M_PI * M_PI, 2.0 / 3.0);
        for (int i = 0; i < neta; ++i) y[i] = lindhard(eta[i], c.lwt_x, 1.0) * factor;
    } else {
        const int sym = c.lwt_kernel == OFDFT_LWT_KERNEL_MGPA ? 1 : (c.lwt_kernel == OFDFT_LWT_KERNEL_MGPG ? 2 : 0);
        y = mgp_kernel_table(eta, c.lwt_maxpoints, sym);
    }
    upload_table<T>(e, eta, y);
}

GgaSpec gga_spec(const ofdft_config& c) {
    GgaSpec s;
    s.formula = c.gga_formula;
    s.np = c.gga_nparams;
    for (int i = 0; i < 8; ++i) s.p[i] = i < c.gga_nparams ? c.gga_params[i] : 0.0;
    s.remove_vw = c.gga_remove_vw;
    s.sigma = c.gga_sigma;
    s.meta = c.gga_formula >= OFDFT_GGA_GE2 ? 1 : 0;
    return s;
}

template <typename T>
Table<T> table_of(const ofdft_eval* e) {
    Table<T> t;
    t.c = (const T*)e->tab_c;
    t.cd = (const T*)e->tab_cd;
    t.nint = e->tab_nint;
    t.step = e->tab_step;
    t.inv_step = 1.0 / e->tab_step;
    t.etamax = e->cfg.lwt_etamax;
    t.limit = e->tab_limit;
    t.limitd = e->tab_limitd;
    t.factor = 4.0 / 5.0 * 0.3 * std::pow(3.0 * M_PI * M_PI, 2.0 / 3.0);
    t.lbda = e->cfg.lwt_x;
    // the large-eta series is the inverse Lindhard function's: WT tables only
    t.eta_series = e->cfg.lwt_kernel == OFDFT_LWT_KERNEL_WT ? 2.5 : INFINITY;
    t.hc = e->cfg.lwt_family == OFDFT_LWT_FAMILY_HC ? 1 : 0;
    return t;
}

struct LwtPlan {
    bool active = false;  // false: homogeneous density, NL term is zero
    std::vector<double> nodes;
    double kfclip = INFINITY;
};

// ------------------------------------------------ fused k_F-node pipeline (host)
constexpr int kFzMaxNodes = 1024;  // node bounds (6 floats each) staged in shared memory
constexpr int kFzMaxBatch = 256;   // node reciprocals staged in shared memory

bool fz_applies(const ofdft_grid* g, int m) {
    auto p2 = [](int n, int lo, int hi) { return n >= lo && n <= hi && (n & (n - 1)) == 0; };
    return g->prec == OFDFT_F32 && m <= kFzMaxNodes && p2(g->nr[0], 32, 256) && p2(g->nr[1], 32, 256) &&
           p2(g->nr[2], 32, 512);
}

// column lengths (axes 0 and 1)
template <class F>
void with_col(int n, F&& f) {
    switch (n) {
        case 32: f(std::integral_constant<int, 32>()); break;
        case 64: f(std::integral_constant<int, 64>()); break;
        case 128: f(std::integral_constant<int, 128>()); break;
        case 256: f(std::integral_constant<int, 256>()); break;
        default: OFDFT_REQUIRE(false, "tile FFT: no column transform of length %d", n);
    }
}

// half lengths of the contiguous axis
template <class F>
void with_row(int h, F&& f) {
    switch (h) {
        case 16: f(std::integral_constant<int, 16>()); break;
        case 32: f(std::integral_constant<int, 32>()); break;
        case 64: f(std::integral_constant<int, 64>()); break;
        case 128: f(std::integral_constant<int, 128>()); break;
        case 256: f(std::integral_constant<int, 256>()); break;
        default: OFDFT_REQUIRE(false, "tile FFT: no row transform of half length %d", h);
    }
}

// exp(-2 pi i k/n) tables for n0, n1, n2/2 and the n2 real-transform twiddles,
// from float64 host trigonometry
void fz_tables(ofdft_eval* e) {
    if (e->fz_tw) return;
    const ofdft_grid* g = e->g;
    const int n0 = g->nr[0], n1 = g->nr[1], n2 = g->nr[2], H = n2 / 2;
    std::vector<float2> h((size_t)n0 + n1 + 2 * (size_t)H + 32);
    auto fill = [&](size_t off, int count, int n) {
        for (int k = 0; k < count; ++k) {
            const double a = -2.0 * M_PI * (double)k / (double)n;
            h[off + k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
    };
    fill(0, n0, n0);
    fill((size_t)n0, n1, n1);
    fill((size_t)n0 + n1, H, H);
    fill((size_t)n0 + n1 + H, H, n2);
    fill((size_t)n0 + n1 + 2 * (size_t)H, 32, 32);  // the 32-point stage of the split path
    OFDFT_CK(cudaMalloc(&e->fz_tw, h.size() * sizeof(float2)));
    upload_now(e->fz_tw, h.data(), h.size() * sizeof(float2));
    OFDFT_CK(cudaMalloc(&e->d_fz_err, sizeof(unsigned)));
    OFDFT_CK(cudaMallocHost(&e->h_fz_err, sizeof(unsigned)));
    *e->h_fz_err = 0;
    upload_now(e->d_fz_err, e->h_fz_err, sizeof(unsigned));
    OFDFT_CK(cudaStreamCreateWithFlags(&e->fz_st2, cudaStreamNonBlocking));
    OFDFT_CK(cudaEventCreateWithFlags(&e->fz_fork, cudaEventDisableTiming));
    OFDFT_CK(cudaEventCreateWithFlags(&e->fz_join, cudaEventDisableTiming));
}

struct FzRun {
    const float2* rbG;  // FFT(rho^beta), half grid
    const float* kf;
    const float* rA;    // rho^alpha
    float* pot1;
    float* pot3;
    float2* pot2G;
    Table<float> tab;
    Nodes nd;
    int m, kdd;
    bool hermite;  // cubic Hermite interpolation (else linear)
    double kfclip;
};

// Dynamic shared memory above the default 48 KB needs a per-kernel opt-in.
template <class K>
void fz_smem_optin(K kernel, size_t bytes) {
    if (bytes > 48 * 1024) OFDFT_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

// Runs every node batch of the fused pipeline; returns the number of launches.
int fz_run(ofdft_eval* e, const FzRun& r, cudaStream_t st) {
    ofdft_grid* g = e->g;
    const ofdft_config& c = e->cfg;
    const int n0 = g->nr[0], n1 = g->nr[1], n2 = g->nr[2], H = n2 / 2;
    fz_tables(e);
    FzDims d;
    d.n0 = n0;
    d.n1 = n1;
    d.n2 = n2;
    d.H = H;
    d.nyq = (long long)n0 * n1 * H;
    d.plane = g->Nc;
    FzTw tw;
    tw.t0 = e->fz_tw;
    tw.t1 = e->fz_tw + n0;
    tw.th = e->fz_tw + n0 + n1;
    tw.tr = e->fz_tw + n0 + n1 + H;
    tw.tq = e->fz_tw + n0 + n1 + 2 * H;
    const FzTab tb = fz_tab(r.tab);
    // the C2R chain with axis 1 split between its two passes (no axis-1 plane pass)
    const bool split = e->cfg.lwt_pipeline == OFDFT_LWT_PIPE_FUSED_SPLIT;
    const size_t cb = g->cplx_bytes();
    // M planes: pot3 (kdd = 3), and pot1 with the Hermite interpolation
    const bool mc = r.kdd == 3 || r.hermite;
    OFDFT_REQUIRE(!(split && r.hermite), "FUSED_SPLIT k_F-node pipeline: linear interpolation only");
    // hat planes per node of the R2C chain: one, two with the Hermite interpolation
    const int hp = r.kdd > 1 ? (r.hermite ? 2 : 1) : 0;
    // planes per node: P (and M) for the C2R chain, hp more for the R2C chain,
    // which runs on a second stream at the same time and needs its own planes
    const int per_node = (mc ? 2 : 1) + hp;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    int B = c.lwt_max_batch > 0 ? c.lwt_max_batch : 64;
    B = std::min(B, kFzMaxBatch);
    const long long fit = (long long)(0.5 * (double)freeb) / (long long)(per_node * cb);
    if (fit < B) B = (int)std::max(1LL, fit);
    B = std::min(B, r.m);
    float2* XY = (float2*)e->sc.get("lwtXY", (size_t)(mc ? 2 : 1) * B * cb);
    float2* XY2 = r.kdd > 1 ? (float2*)e->sc.get("lwtXY2", (size_t)hp * B * cb) : nullptr;
    // the R2C chain (hat planes -> pot2) does not depend on the C2R chain (node
    // planes -> pot1/pot3): fork it onto the second stream, join before return.
    // With per-kernel profiling on, both chains stay on st so that each
    // kernel's events time that kernel alone.
    const bool two = r.kdd > 1 && !e->prof;
    cudaStream_t st2 = two ? e->fz_st2 : st;
    if (two) {
        OFDFT_CK(cudaEventRecord(e->fz_fork, st));
        OFDFT_CK(cudaStreamWaitEvent(st2, e->fz_fork, 0));
    }
    const double Ncd = (double)g->Nc, Nd = (double)g->N;
    const float invN = (float)(1.0 / Nd);
    const int tiles0 = n1 * (H / kFzLines) + n1 / kFzLines;
    const int tiles1 = n0 * (H / kFzLines) + n0 / kFzLines;
    const double* knode = r.nd.k;
    const double* invk = r.nd.invk;
    int launches = 0;
    for (int j0 = 0; j0 < r.m; j0 += B) {
        const int nb = std::min(B, r.m - j0);
        const int nplanes = mc ? 2 * nb : nb;
        const bool first = j0 == 0;
        // ---- C2R: axis 0 with the node kernels applied on load (P planes, then M
        // planes); nodes split over blocks when the tile count alone leaves a long
        // last wave
        const int nsplit = (nb >= 16 && tiles0 < 8 * g->sms) ? 2 : 1;
        FzRowArgs ra;
        ra.kf = r.kf;
        ra.rA = r.rA;
        ra.XY = XY;
        ra.pot1 = r.pot1;
        ra.pot3 = r.pot3;
        ra.kn = e->d_nodes;
        ra.kup = e->d_nodes + 2 * kMaxNodes;
        ra.m = r.m;
        ra.j0 = j0;
        ra.nb = nb;
        ra.first = first ? 1 : 0;
        ra.kfclip = r.kfclip;
        ra.d = d;
        ra.tw = tw;
        ra.err = e->d_fz_err;
        if (split) {
            // axis 0 + the radix-8 stage of axis 1, then the 32-point stage with the rows
            with_col(n0, [&](auto c0) {
                constexpr int N0 = decltype(c0)::value;
                const size_t smem = fz8_nodes_smem(N0, nb);
                auto launch = [&](auto kern, int plane0) {
                    fz_smem_optin(kern, smem);
                    timed(e, P_LWT_NODES, Ncd * 8.0 * (1 + nb), st, [&] {
                        kern<<<fz8_tiles(H), kS8L * (N0 / kFzColE), smem, st>>>(
                            r.rbG, XY, tb, knode, invk, j0, nb, plane0, g->geo, d, tw.t0, tw.t1, invN);
                    });
                    OFDFT_LAUNCH_CHECK();
                };
                launch(k_fz_n8<N0, false>, 0);
                if (mc) launch(k_fz_n8<N0, true>, nb);
            });
            const size_t smem = fz8_row_smem(r.m, 2);
            const int grid = n0 * 8;
            auto launch = [&](auto kern, int plane0, float* pot) {
                fz_smem_optin(kern, smem);
                timed(e, P_LWT_INTERP, Ncd * 8.0 * nb + Nd * 4.0 * (1 + (first ? 1 : 2)), st,
                      [&] { kern<<<grid, kS8RowThreads, smem, st>>>(ra, plane0, pot); });
                OFDFT_LAUNCH_CHECK();
            };
            launch(k_fz_c2r_s8<true>, 0, r.pot1);
            if (mc) launch(k_fz_c2r_s8<false>, nb, r.pot3);
            launches += mc ? 4 : 2;
        }
        if (!split) with_col(n0, [&](auto c0) {
            constexpr int N0 = decltype(c0)::value;
            const size_t smem = fz_col_smem(N0, nb, true);
            auto launch = [&](auto kern, int plane0) {
                fz_smem_optin(kern, smem);
                timed(e, P_LWT_NODES, Ncd * 8.0 * (nsplit + nb), st, [&] {
                    kern<<<tiles0 * nsplit, kFzLines * (N0 / kFzColE), smem, st>>>(
                        r.rbG, XY, tb, knode, invk, j0, nb, plane0, tiles0, nsplit, g->geo, d, tw.t0, invN);
                });
                OFDFT_LAUNCH_CHECK();
            };
            launch(k_fz_nodes<N0, false>, 0);
            if (mc) launch(k_fz_nodes<N0, true>, nb);
        });
        // ---- axis 1
        if (!split) with_col(n1, [&](auto c1) {
            constexpr int N1 = decltype(c1)::value;
            const size_t smem = std::max(fz::col_slots(N1), kFzLines * fz::row_slots(N1)) * sizeof(float2);
            timed(e, P_FZ_AXIS1, Ncd * 16.0 * nplanes, st,
                  [&] { k_fz_axis1<N1, +1><<<tiles1 * nplanes, N1, smem, st>>>(XY, d, tw.t1); });
        });
        OFDFT_LAUNCH_CHECK();
        // ---- axis 2 C2R with the interpolation into pot1 (pot3)
        if (!split) with_row(H, [&](auto ch) {
            constexpr int HH = decltype(ch)::value;
            constexpr int ROWS = kFzRowThreads / (HH / kFzRowE);
            const size_t smem = fz_row_smem(HH, r.m, true);
            const int grid = (int)((long long)n0 * n1 / ROWS);
            auto launch = [&](auto kern, int plane0, float* pot) {
                fz_smem_optin(kern, smem);
                timed(e, P_LWT_INTERP, Ncd * 8.0 * nb + Nd * 4.0 * (1 + (first ? 1 : 2)), st,
                      [&] { kern<<<grid, kFzRowThreads, smem, st>>>(ra, plane0, pot); });
                OFDFT_LAUNCH_CHECK();
            };
            if (r.hermite) {
                // P and M planes both feed pot1 and pot3
                launch(k_fz_c2r_rows<HH, true, 1>, 0, r.pot1);
                launch(k_fz_c2r_rows<HH, false, 2>, nb, r.pot1);
            } else {
                launch(k_fz_c2r_rows<HH, true>, 0, r.pot1);
                if (mc) launch(k_fz_c2r_rows<HH, false>, nb, r.pot3);
            }
        });
        if (!split) launches += mc ? 5 : 3;
        if (r.kdd > 1) {
            // ---- R2C on the second stream: hat-weighted rho^alpha along axis 2, then axis 1,
            // then axis 0 into pot2(G)
            FzRowArgs ra2 = ra;
            ra2.XY = XY2;
            if (split) {
                // hat weights, axis 2 and the 32-point stage of axis 1; then the
                // radix-8 stage, axis 0 and the sum into pot2(G)
                const size_t smem = fz8_row_smem(r.m, 1);
                fz_smem_optin(k_fz_r2c_s8, smem);
                timed(e, P_FZ_HAT, Nd * 8.0 + Ncd * 8.0 * nb, st2,
                      [&] { k_fz_r2c_s8<<<n0 * 8, kS8RowThreads, smem, st2>>>(ra2); });
                OFDFT_LAUNCH_CHECK();
                with_col(n0, [&](auto c0) {
                    constexpr int N0 = decltype(c0)::value;
                    const size_t smem0 = fz8_pot2_smem(N0, nb);
                    fz_smem_optin(k_fz_pot2_s8<N0>, smem0);
                    timed(e, P_LWT_POT2, Ncd * 8.0 * (nb + (first ? 1 : 2)), st2, [&] {
                        k_fz_pot2_s8<N0><<<fz8_tiles(H), kS8L * (N0 / kFzColE), smem0, st2>>>(
                            XY2, r.pot2G, tb, knode, invk, j0, nb, first ? 1 : 0, g->geo, d, tw.t0, invN);
                    });
                });
                OFDFT_LAUNCH_CHECK();
                launches += 2;
            }
            if (!split) with_row(H, [&](auto ch) {
                constexpr int HH = decltype(ch)::value;
                constexpr int ROWS = kFzRowThreads / (HH / kFzRowE);
                const size_t smem = fz_row_smem(HH, r.m, false);
                const int grid = (int)((long long)n0 * n1 / ROWS);
                auto hat = [&](auto kern) {
                    fz_smem_optin(kern, smem);
                    timed(e, P_FZ_HAT, Nd * 8.0 + Ncd * 8.0 * hp * nb, st2,
                          [&] { kern<<<grid, kFzRowThreads, smem, st2>>>(ra2); });
                };
                if (r.hermite) hat(k_fz_r2c_rows<HH, true>);
                else hat(k_fz_r2c_rows<HH>);
            });
            OFDFT_LAUNCH_CHECK();
            if (!split) with_col(n1, [&](auto c1) {
                constexpr int N1 = decltype(c1)::value;
                const size_t smem = std::max(fz::col_slots(N1), kFzLines * fz::row_slots(N1)) * sizeof(float2);
                timed(e, P_FZ_AXIS1, Ncd * 16.0 * hp * nb, st2,
                      [&] { k_fz_axis1<N1, -1><<<tiles1 * hp * nb, N1, smem, st2>>>(XY2, d, tw.t1); });
            });
            OFDFT_LAUNCH_CHECK();
            if (!split) with_col(n0, [&](auto c0) {
                constexpr int N0 = decltype(c0)::value;
                const size_t smem = fz_col_smem(N0, nb, false);
                auto pot2 = [&](auto kern) {
                    fz_smem_optin(kern, smem);
                    timed(e, P_LWT_POT2, Ncd * 8.0 * (hp * nb + (first ? 1 : 2)), st2, [&] {
                        kern<<<tiles0, kFzLines * (N0 / kFzColE), smem, st2>>>(
                            XY2, r.pot2G, tb, knode, invk, j0, nb, first ? 1 : 0, g->geo, d, tw.t0, invN);
                    });
                };
                if (r.hermite) pot2(k_fz_pot2<N0, true>);
                else pot2(k_fz_pot2<N0>);
            });
            OFDFT_LAUNCH_CHECK();
            if (!split) launches += 3;
        }
    }
    if (two) {
        OFDFT_CK(cudaEventRecord(e->fz_join, st2));
        OFDFT_CK(cudaStreamWaitEvent(st, e->fz_join, 0));
    }
    return launches;
}

void collect_energies(ofdft_eval* e, double* energies);

// Enqueues one evaluation on st.  With energies != NULL it waits for the
// stream and writes them; with NULL it returns after enqueueing the copy of
// the sums to the grid's pinned results, and collect_energies() reads them
// once the caller has synchronised the stream.
template <typename T>
void compute_t(ofdft_eval* e, const T* rho, T* V, unsigned calc, double* energies, cudaStream_t st) {
    ofdft_grid* g = e->g;
    const ofdft_config& c = e->cfg;
    const long long N = g->N, Nc = g->Nc;
    const bool wantV = (calc & OFDFT_CALC_V) != 0;
    const bool tf = c.kedf_terms & OFDFT_KE_TF, vw = c.kedf_terms & OFDFT_KE_VW;
    const bool wt = c.kedf_terms & OFDFT_KE_WT, lwt = c.kedf_terms & OFDFT_KE_LWT;
    const bool hc = lwt && c.lwt_family == OFDFT_LWT_FAMILY_HC;
    OFDFT_REQUIRE(!lwt || e->tab_set, "k_F-node kernel: no table set (ofdft_eval_set_lwt_table)");
    const bool nl = wt || lwt;
    const double alpha = wt ? c.wt_alpha : c.lwt_alpha, beta = wt ? c.wt_beta : c.lwt_beta;
    const bool same_ab = wt ? std::fabs(beta - alpha) < 1e-9 : std::fabs(alpha - beta) < 1e-8;
    const bool h = c.hartree != 0, xc = c.xc_lda != 0, pp = c.pseudo != 0 && e->have_vloc;
    const bool wte = c.wte != 0 && tf && wt;  // WTE scales the TF and WT potentials after the sums
    OFDFT_REQUIRE(!(c.pseudo && !e->have_vloc), "ofdft_eval_compute: pseudo enabled but no v_loc set");
    const bool ext = c.external != 0;
    OFDFT_REQUIRE(!(ext && !e->have_vext), "ofdft_eval_compute: external potential enabled but not set");
    OFDFT_REQUIRE(!(wantV && !V), "ofdft_eval_compute: V requested but v_out is NULL");
    int launches = 0;
    const size_t rb = g->real_bytes(), cb = g->cplx_bytes();
    using C = typename Cplx<T>::type;

    T* Vw = wantV ? V : nullptr;
    T* sq = vw ? (T*)e->sc.get("sq", rb) : nullptr;
    T* rbp = nl ? (T*)e->sc.get("rb", rb) : nullptr;
    T* rap = (nl && !same_ab) ? (T*)e->sc.get("ra", rb) : nullptr;
    T* kfv = lwt ? (T*)e->sc.get("kf", rb) : nullptr;

    // ---- pre-pass
    PreArgs<T> pa;
    pa.rho = rho;
    pa.vloc = pp ? (const T*)e->vloc : nullptr;
    pa.vext = ext ? (const T*)e->vext : nullptr;
    pa.V = Vw;
    pa.sq = sq;
    pa.rb = rbp;
    pa.ra = rap;
    pa.kf = kfv;
    pa.N = N;
    pa.tf = tf;
    pa.tf_v = !wte;
    pa.dttf = (c.kedf_terms & OFDFT_KE_DTTF) != 0;
    pa.dttf_old = c.tf_temp_old;
    pa.temp = c.tf_temperature;
    pa.vw = vw;
    pa.xc = xc;
    pa.pp = pp;
    pa.ext = ext;
    pa.nl = nl;
    pa.lwt = lwt && !hc;  // HC builds its k_F from the gradient below
    pa.same_ab = same_ab;
    pa.wantV = wantV;
    pa.nl_is_lwt = lwt && !hc;  // HC clamps rho at 1e-30 as WT does (hc.py:88-90)
    pa.tf_x = c.tf_x;
    pa.alpha = alpha;
    pa.beta = beta;
    pa.k = e->k;
    const double s = (double)sizeof(T), Nd = (double)N, Ncd = (double)Nc;
    {
        // algorithmic bytes: read rho (+ v_loc); write V, sqrt(rho), rho^beta (+ rho^alpha), k_F as active
        double b = Nd * s * (1 + pp + ext + wantV + vw + nl + (nl && !same_ab) + lwt);
        timed(e, P_PREPASS, b, st, [&] { k_prepass<T><<<g->red_blocks, RED_THREADS, 0, st>>>(pa, g->d_partials); });
    }
    OFDFT_LAUNCH_CHECK();
    unsigned long long kinds = (1ull << (2 * 4)) | (2ull << (2 * 5)) | (2ull << (2 * 6));
    timed(e, P_REDUCE, (double)g->red_blocks * PRE_NS * 8, st, [&] {
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, PRE_NS, kinds, g->d_results);
    });
    OFDFT_LAUNCH_CHECK();
    launches += 2;
    auto r2c = [&](const void* in, void* out, int batch) {
        timed(e, P_CUFFT, 2.0 * Nd * s * batch, st, [&] { g->exec_r2c(in, out, batch, st); });
    };
    auto c2r = [&](void* in, void* out, int batch) {
        timed(e, P_CUFFT, 2.0 * Nd * s * batch, st, [&] { g->exec_c2r(in, out, batch, st); });
    };

    // ---- WT kernel cache decision on the device
    T* wtK = nullptr;
    if (wt) {
        wtK = (T*)e->sc.get("wtK", (size_t)Nc * sizeof(T));
        k_wt_plan<<<1, 1, 0, st>>>(g->d_results, e->wtstate, c.wt_rho0, 1.0 / (double)N, c.wt_alpha, c.wt_beta,
                                   e->k.cTF_wt);
        OFDFT_LAUNCH_CHECK();
        launches++;
        if (c.wt_kernel != OFDFT_LWT_KERNEL_WT) {  // MGP kernel at rho0, rebuilt when k_wt_plan says so
            MgpArgs m;
            m.x = e->mgp_x;
            m.c = e->mgp_c;
            m.n = e->mgp_n;
            m.maxpoints = c.wt_maxpoints;
            m.sym = c.wt_kernel == OFDFT_LWT_KERNEL_MGPA ? 1 : (c.wt_kernel == OFDFT_LWT_KERNEL_MGPG ? 2 : 0);
            m.lump = c.wt_lump;
            for (int k = 0; k < 3; ++k) m.abc[k] = c.wt_lump_abc[k];
            m.revke = c.wt_revke;
            m.volume = g->volume;
            const int nb = blocks_for(Nc, 128, g->sms * 8);
            k_mgp_kernel<T><<<nb, 128, 0, st>>>(wtK, g->geo, e->wtstate, m);
            OFDFT_LAUNCH_CHECK();
            launches++;
        }
    }

    // ---- HC: k_F = F(s) (3 pi^2 rho)^(1/3) from the gradient of the clamped density
    T *hcD = nullptr, *hc_c1 = nullptr, *hc_c2 = nullptr;
    C* hcX = nullptr;
    C* hcG = nullptr;
    if (hc) {
        const int gblk = blocks_for(Nc, 256, g->sms * 16), rblk = blocks_for(N, 256, g->sms * 16);
        T* rc = (T*)e->sc.get("hc_rc", rb);
        hcG = (C*)e->sc.get("hc_G", cb);
        hcX = (C*)e->sc.get("hc_X", 3 * cb);
        hcD = (T*)e->sc.get("hc_D", 3 * rb);
        if (wantV) {
            hc_c1 = (T*)e->sc.get("hc_c1", rb);
            hc_c2 = (T*)e->sc.get("hc_c2", rb);
        }
        k_hc_clamp<T><<<rblk, 256, 0, st>>>(rho, rc, N);
        OFDFT_LAUNCH_CHECK();
        r2c(rc, hcG, 1);
        k_grad_spectra<T><<<gblk, 256, 0, st>>>(hcG, hcX, g->geo, 1.0 / (double)N, 0.0, 0);
        OFDFT_LAUNCH_CHECK();
        c2r(hcX, hcD, 3);
        k_hc_point<T><<<g->red_blocks, RED_THREADS, 0, st>>>(rho, hcD, kfv, hc_c1, hc_c2, N, gga_spec(c),
                                                             g->d_partials);
        OFDFT_LAUNCH_CHECK();
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 2, (1ull << 0) | (2ull << 2),
                                                   g->d_results + 48);
        OFDFT_LAUNCH_CHECK();
        launches += 5;
    }

    // ---- k_F node plan on the host (needs min/max k_F and max rho)
    LwtPlan lp;
    double rhomax = 0.0;
    if (hc) {  // get_kflist (hc.py:144-158): nodes first (the state moves), then the HEG test
        OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, 50 * sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        const double kf_l = g->h_results[48], kf_r = g->h_results[49];
        rhomax = g->h_results[6];
        const bool fmin_ = !std::isnan(c.lwt_kfmin), fmax_ = !std::isnan(c.lwt_kfmax);
        lp.nodes = hc_kf_nodes(kf_l, kf_r, fmin_, c.lwt_kfmin, fmax_, c.lwt_kfmax, e->kf_set_min, e->kf_st_min,
                               e->kf_set_max, e->kf_st_max, c.lwt_ratio, c.lwt_nsp, c.lwt_delta);
        const int m = (int)lp.nodes.size();
        lp.active = !(std::fabs(kf_r - kf_l) < 1e-8 || m < 3);
        if (lp.active) {
            OFDFT_REQUIRE(m <= kMaxNodes, "density-dependent kernel: %d nodes (max %d)", m, kMaxNodes);
            lp.kfclip = lp.nodes.back();
            for (int i = 0; i < m; ++i) {
                e->h_nodes[i] = lp.nodes[i];
                e->h_nodes[kMaxNodes + i] = 1.0 / (2.0 * lp.nodes[i]);  // HCKernelXi: xi = 2k
                e->h_nodes[2 * kMaxNodes + i] = lp.nodes[i] + 1e-18;
            }
            OFDFT_CK(cudaMemcpyAsync(e->d_nodes, e->h_nodes, 3 * kMaxNodes * sizeof(double), cudaMemcpyHostToDevice,
                                     st));
        }
        e->last_nsp = lp.active ? m : 0;
    } else if (lwt) {
        OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, PRE_NS * sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        const double kf_l = g->h_results[4], kf_r = g->h_results[5];
        rhomax = g->h_results[6];
        if (std::fabs(kf_r - kf_l) >= 1e-8) {  // lwt.py:115-124
            lp.active = true;
            const bool fmin_ = !std::isnan(c.lwt_kfmin), fmax_ = !std::isnan(c.lwt_kfmax);
            double b0, b1;
            guess_kf_bound(kf_l, kf_r, fmin_, c.lwt_kfmin, fmax_, c.lwt_kfmax, e->kf_set_min, e->kf_st_min,
                           e->kf_set_max, e->kf_st_max, b0, b1);
            lp.kfclip = b1;
            double kmin_c = std::min(kf_l, b1), kmax_c = std::min(kf_r, b1);
            double kfMin = fmin_ ? c.lwt_kfmin : std::max(kmin_c, b0);
            double kfMax = fmax_ ? c.lwt_kfmax : kmax_c;
            lp.nodes = kf_nodes(kfMin, kfMax, c.lwt_nsp, c.lwt_delta, c.lwt_ratio);
            OFDFT_REQUIRE((int)lp.nodes.size() <= kMaxNodes && lp.nodes.size() >= 2,
                          "density-dependent kernel: %zu nodes (max %d)", lp.nodes.size(), kMaxNodes);
            const int m = (int)lp.nodes.size();
            for (int i = 0; i < m; ++i) {
                e->h_nodes[i] = lp.nodes[i];
                e->h_nodes[kMaxNodes + i] = 1.0 / lp.nodes[i];
                e->h_nodes[2 * kMaxNodes + i] = lp.nodes[i] + 1e-18;
            }
            OFDFT_CK(cudaMemcpyAsync(e->d_nodes, e->h_nodes, 3 * kMaxNodes * sizeof(double), cudaMemcpyHostToDevice,
                                     st));
        }
        e->last_nsp = lp.active ? (int)lp.nodes.size() : 0;
    }

    // ---- forward transforms
    C* rhoG = h ? (C*)e->sc.get("rhoG", cb) : nullptr;
    C* sqG = vw ? (C*)e->sc.get("sqG", cb) : nullptr;
    C* rbG = nl ? (C*)e->sc.get("rbG", cb) : nullptr;
    C* raG = (wt && !same_ab) ? (C*)e->sc.get("raG", cb) : nullptr;
    if (h) r2c(rho, rhoG, 1);
    if (vw) r2c(sq, sqG, 1);
    if (wt || (lwt && lp.active)) r2c(rbp, rbG, 1);
    if (raG) r2c(rap, raG, 1);

    // ---- fused G-space multipliers
    if (h || vw || wt) {
        GArgs<T> ga;
        ga.rhoG = rhoG;
        ga.sqG = sqG;
        ga.rbG = wt ? rbG : nullptr;
        ga.raG = raG;
        ga.wtK = wtK;
        ga.mgp = c.wt_kernel != OFDFT_LWT_KERNEL_WT;
        ga.wtstate = e->wtstate;
        ga.wt_x = c.wt_x;
        ga.vw_s = c.vw_sigma > 0.0 ? c.vw_sigma * c.vw_sigma / 4.0 : 0.0;
        ga.geo = g->geo;
        ga.invN = 1.0 / (double)N;
        // read + write of each active complex plane (+ the cached WT kernel)
        double b = Ncd * 2 * s * 2 * (h + vw + wt + (raG != nullptr)) + (wt ? Ncd * s : 0.0);
        timed(e, P_GSPACE, b, st, [&] { k_gspace<T><<<blocks_for(Nc, 256, g->sms * 16), 256, 0, st>>>(ga); });
        OFDFT_LAUNCH_CHECK();
        launches++;
    }
    T* vH = h ? (T*)e->sc.get("vH", rb) : nullptr;
    T* lap = vw ? (T*)e->sc.get("lap", rb) : nullptr;
    T* nl1 = wt ? (T*)e->sc.get("nl1", rb) : nullptr;
    T* nl2 = (wt && !same_ab) ? (T*)e->sc.get("nl2", rb) : nullptr;
    if (h) c2r(rhoG, vH, 1);
    if (vw) c2r(sqG, lap, 1);
    if (wt) c2r(rbG, nl1, 1);
    if (nl2) c2r(raG, nl2, 1);

    // ---- density-dependent kernel
    T *pot1 = nullptr, *pot2 = nullptr, *pot3 = nullptr;
    int kdd = wantV ? (hc ? 3 : c.lwt_kdd) : 1;  // HC keeps every derivative term
    if (lwt && lp.active) {
        const int m = (int)lp.nodes.size();
        const bool hermite = c.lwt_interp == OFDFT_INTERP_HERMITE;
        const bool mcalc = kdd > 1 || hermite;
        pot1 = (T*)e->sc.get("pot1", rb);
        if (kdd == 3) pot3 = (T*)e->sc.get("pot3", rb);
        C* pot2G = kdd > 1 ? (C*)e->sc.get("pot2G", cb) : nullptr;
        Nodes nd;
        nd.k = e->d_nodes;
        nd.invk = e->d_nodes + kMaxNodes;
        bool fused = false;
        if (c.lwt_pipeline != OFDFT_LWT_PIPE_CUFFT) {
            fused = c.lwt_family == OFDFT_LWT_FAMILY_LWT && fz_applies(g, m);
            OFDFT_REQUIRE(c.lwt_pipeline != OFDFT_LWT_PIPE_FUSED_SPLIT || (g->nr[1] == 256 && g->nr[2] == 256),
                          "FUSED_SPLIT k_F-node pipeline: needs n1 = n2 = 256");
            OFDFT_REQUIRE(fused || (c.lwt_pipeline != OFDFT_LWT_PIPE_FUSED && c.lwt_pipeline != OFDFT_LWT_PIPE_FUSED_SPLIT),
                          "fused k_F-node pipeline: needs a float32 grid, at most %d nodes and "
                          "power-of-two axes (32..256, the last 32..512)",
                          kFzMaxNodes);
        }
        if constexpr (std::is_same<T, float>::value) {
            if (fused) {
                FzRun fr;
                fr.rbG = rbG;
                fr.kf = kfv;
                fr.rA = same_ab ? rbp : rap;
                fr.pot1 = pot1;
                fr.pot3 = pot3;
                fr.pot2G = pot2G;
                fr.tab = table_of<float>(e);
                fr.nd = nd;
                fr.m = m;
                fr.kdd = kdd;
                fr.hermite = hermite;
                fr.kfclip = lp.kfclip;
                launches += fz_run(e, fr, st);
                e->fz_ran = true;
            }
        }
        if (!fused) {
            // nodes per batched pass from the free memory: per node 2 complex + 2 real + (1|2) real planes
            size_t per_node = 2 * cb + 2 * rb + (hermite ? 2 : 1) * rb;
            size_t freeb = 0, totalb = 0;
            cudaMemGetInfo(&freeb, &totalb);
            int B = c.lwt_max_batch > 0 ? c.lwt_max_batch : 64;
            long long fit = (long long)(0.5 * (double)freeb) / (long long)per_node;
            if (fit < B) B = (int)std::max(1LL, fit);
            B = std::min(B, m);
            C* XY = (C*)e->sc.get("lwtXY", (size_t)2 * B * cb);
            T* PM = (T*)e->sc.get("lwtPM", (size_t)2 * B * rb);
            T* U = kdd > 1 ? (T*)e->sc.get("lwtU", (size_t)(hermite ? 2 : 1) * B * rb) : nullptr;
            Table<T> tab = table_of<T>(e);
            const int gblk = blocks_for(Nc, 256, g->sms * 16);
            const int rblk = blocks_for(N, 256, g->sms * 16);
            for (int j0 = 0; j0 < m; j0 += B) {
                const int nb = std::min(B, m - j0);
                const int nplanes = mcalc ? 2 * nb : nb;
                // read FFT(rho^beta) once, write one complex plane per node (two with derivatives)
                timed(e, P_LWT_NODES, Ncd * 2 * s * (1 + nplanes), st, [&] {
                    k_lwt_nodes<T><<<gblk, 256, nb * sizeof(T), st>>>(rbG, XY, tab, nd, j0, nb, mcalc, g->geo,
                                                                     1.0 / (double)N);
                });
                OFDFT_LAUNCH_CHECK();
                c2r(XY, PM, nplanes);
                InterpArgs<T> ia;
                ia.kf = kfv;
                ia.rA = same_ab ? rbp : rap;
                ia.PM = PM;
                ia.pot1 = pot1;
                ia.pot3 = pot3;
                ia.u = U;
                ia.kn = e->d_nodes;
                ia.kup = e->d_nodes + 2 * kMaxNodes;
                ia.m = m;
                ia.j0 = j0;
                ia.nb = nb;
                ia.kdd = kdd;
                ia.hermite = hermite;
                ia.mcalc = mcalc;
                ia.first = j0 == 0;
                ia.kfclip = lp.kfclip;
                ia.N = N;
                {
                    // read k_F and rho^alpha; gather the two (four with derivatives) node values of each
                    // point; write pot1 (+pot3), reading them back after the first pass; write the hat planes
                    const int upl = kdd > 1 ? (hermite ? 2 * nb : nb) : 0;
                    const int gat = kdd == 3 || hermite ? 4 : 2;
                    const int accs = 1 + (kdd == 3);
                    double b = Nd * s * (2 + gat + accs * (j0 == 0 ? 1 : 2) + upl);
                    timed(e, P_LWT_INTERP, b, st,
                          [&] { k_lwt_interp<T><<<rblk, 256, 2 * m * sizeof(double), st>>>(ia); });
                }
                OFDFT_LAUNCH_CHECK();
                launches += 2;
                if (kdd > 1) {
                    const int upl = hermite ? 2 * nb : nb;
                    r2c(U, XY, upl);
                    timed(e, P_LWT_POT2, Ncd * 2 * s * (upl + (j0 == 0 ? 1 : 2)), st, [&] {
                        k_lwt_pot2<T><<<gblk, 256, nb * sizeof(T), st>>>(XY, pot2G, tab, nd, j0, nb, hermite, j0 == 0, g->geo,
                                                             1.0 / (double)N);
                    });
                    OFDFT_LAUNCH_CHECK();
                    launches += 1;
                }
            }
        }
        if (kdd > 1) {
            pot2 = (T*)e->sc.get("pot2", rb);
            c2r(pot2G, pot2, 1);
        }
    }
    // ---- HC: the divergence term of dk_F/d(grad rho) (hc.py:313-318)
    T* hc_q = nullptr;
    if (hc && wantV && lp.active) {
        const int gblk = blocks_for(Nc, 256, g->sms * 16), rblk = blocks_for(N, 256, g->sms * 16);
        k_hc_p<T><<<rblk, 256, 0, st>>>(hcD, hc_c2, same_ab ? rbp : rap, pot3, N);
        OFDFT_LAUNCH_CHECK();
        r2c(hcD, hcX, 3);
        k_gga_div<T><<<gblk, 256, 0, st>>>(hcX, hcG, g->geo, 1.0 / (double)N, 0, 0.0);
        OFDFT_LAUNCH_CHECK();
        hc_q = hcD;  // the first gradient plane is free again
        c2r(hcG, hc_q, 1);
        launches += 4;
    }

    // ---- post-pass
    PostArgs<T> qa;
    qa.rho = rho;
    qa.V = Vw;
    qa.Vnl = (wte && wantV) ? (T*)e->sc.get("wte_vnl", rb) : nullptr;
    qa.sq = sq;
    qa.lap = lap;
    qa.vH = vH;
    qa.nl1 = nl1;
    qa.nl2 = nl2;
    qa.rb = rbp;
    qa.ra = rap;
    qa.kf = kfv;
    qa.pot1 = pot1;
    qa.pot2 = pot2;
    qa.pot3 = pot3;
    qa.N = N;
    qa.vw = vw;
    qa.h = h;
    qa.wt = wt;
    qa.lwt = lwt && lp.active;
    qa.same_ab = same_ab;
    qa.wantV = wantV;
    qa.kdd = kdd;
    qa.vw_y = c.vw_y;
    qa.alpha = alpha;
    qa.beta = beta;
    qa.rhomax = rhomax;
    qa.ld = std::max(0.1, c.lwt_ldw);
    qa.kfclip = lp.kfclip;
    qa.hc = hc;
    qa.hc_c1 = hc_c1;
    qa.hc_q = hc_q;
    {
        const bool lw = lwt && lp.active;
        int reads = 1 + wantV + 2 * vw + h + (wt ? 2 + !same_ab * 2 : 0) +
                    (lw ? 1 + 1 + !same_ab + 1 + (kdd > 1) + (kdd == 3) : 0);
        double b = Nd * s * (reads + wantV);
        timed(e, P_POSTPASS, b, st,
              [&] { k_postpass<T><<<g->red_blocks, RED_THREADS, 0, st>>>(qa, g->d_partials); });
    }
    OFDFT_LAUNCH_CHECK();
    timed(e, P_REDUCE, (double)g->red_blocks * POST_NS * 8, st, [&] {
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, POST_NS, 0ull, g->d_results + 16);
    });
    OFDFT_LAUNCH_CHECK();
    launches += 2;
    if (wte && wantV) {  // wte.py:15-18: V += exp(r) ((1 - r) V_TF + V_WT), r = E_WT / E_TF, from the device sums
        const int nb = blocks_for(N, 256, g->sms * 8);
        k_wte_combine<T><<<nb, 256, 0, st>>>(rho, V, qa.Vnl, N, g->d_results, g->d_results + 16, g->dV, c.tf_x,
                                             e->k.cTF_V);
        OFDFT_LAUNCH_CHECK();
        ++launches;
    }
    // ---- GGA kinetic functional: its own gradient and divergence transforms, its
    // potential added to V, its sums in results [40, 48)
    const bool gga = (c.kedf_terms & OFDFT_KE_GGA) != 0;
    if (gga) {
        gga_enqueue<T>(g, e->sc, gga_spec(c), rho, Vw, true, false, g->d_results + 40, st);
        launches += wantV ? 7 : 4;
    }
    OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, (gga ? 48 : 24) * sizeof(double), cudaMemcpyDeviceToHost,
                             st));
    if (e->fz_ran) OFDFT_CK(cudaMemcpyAsync(e->h_fz_err, e->d_fz_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    e->pend.tf = tf;
    e->pend.vw = vw;
    e->pend.wt = wt;
    e->pend.lwt = lwt;
    e->pend.xc = xc;
    e->pend.h = h;
    e->pend.pp = pp;
    e->pend.ext = ext;
    e->pend.lp_active = lwt && lp.active;
    e->pend.gga = gga;
    e->pend.launches = launches;
    if (!energies) return;
    OFDFT_CK(cudaStreamSynchronize(st));
    collect_energies(e, energies);
}

// Energies of the last enqueued evaluation, after its stream has been synchronised.
void collect_energies(ofdft_eval* e, double* energies) {
    const ofdft_config& c = e->cfg;
    const ofdft_eval::Pending& p = e->pend;
    if (e->prof) prof_collect(e);
    if (e->fz_ran) {
        e->fz_ran = false;
        if (*e->h_fz_err) {
            *e->h_fz_err = 0;
            upload_now(e->d_fz_err, e->h_fz_err, sizeof(unsigned));
            OFDFT_REQUIRE(false, "fused k_F-node pipeline: a bulk copy into shared memory did not complete");
        }
    }
    const double* R = e->g->h_results;
    const double dV = e->g->dV;
    double* E = energies;
    for (int i = 0; i < OFDFT_NE; ++i) E[i] = 0.0;
    E[OFDFT_E_TF] = p.tf ? R[0] * dV * c.tf_x : 0.0;
    const double e_wt_raw = p.wt ? R[18] * dV : 0.0;
    E[OFDFT_E_XC] = p.xc ? R[1] * dV : 0.0;
    E[OFDFT_E_PP] = p.pp ? R[2] * dV : 0.0;
    E[OFDFT_E_NELEC] = R[3] * dV;
    E[OFDFT_E_VW] = p.vw ? R[16] * dV * c.vw_y : 0.0;
    E[OFDFT_E_H] = p.h ? R[17] * dV / 2.0 : 0.0;
    if (p.wt) E[OFDFT_E_NL] = R[18] * dV;
    if (p.lwt) E[OFDFT_E_NL] = p.lp_active ? R[18] * dV : 0.0;
    E[OFDFT_E_II] = c.ewald_energy;
    E[OFDFT_E_GGA] = p.gga ? R[40] * dV : 0.0;
    E[OFDFT_E_EXT] = p.ext ? R[7] * dV : 0.0;
    E[OFDFT_E_DTTF] = (c.kedf_terms & OFDFT_KE_DTTF) ? R[8] * dV * c.tf_x : 0.0;
    if (c.wte && p.tf && p.wt) {  // wte.py:20-22
        E[OFDFT_E_NL] = E[OFDFT_E_TF] * std::exp(e_wt_raw / E[OFDFT_E_TF]);
        E[OFDFT_E_TF] = 0.0;
    }
    E[OFDFT_E_TOTAL] = E[OFDFT_E_TF] + E[OFDFT_E_VW] + E[OFDFT_E_NL] + E[OFDFT_E_XC] + E[OFDFT_E_H] + E[OFDFT_E_PP] +
                       E[OFDFT_E_II] + E[OFDFT_E_GGA] + E[OFDFT_E_EXT] + E[OFDFT_E_DTTF];
    e->last_launches = p.launches;
}

// ------------------------------------------------------------------ stress
// Stress tensors of the evaluator's terms (TotalFunctional.get_stress,
// total_functional.py:176-208): TF (kedf/tf.py:52-63), vW (kedf/vw.py:97-111),
// WT (kedf/wt.py:75-106), LDA (xc/semilocal_xc.py:343-346) and Hartree
// (hartree.py:67-90).  Components k = 0..5 are (0,0) (0,1) (0,2) (1,1) (1,2)
// (2,2), the reference's loop order.

// LindhardDerivative(eta, mu) * eta (kedf/kernel.py:197-211); the two
// boundary values eta = 1e-10 and |eta - 1| = 1e-10 fall in no branch (0).
__device__ inline double lindhard_deriv_eta(double eta, double mu) {
    const double atol = 1.0e-10;
    double ld = 0.0;
    if (eta > atol && fabs(eta - 1.0) > atol) {
        const double A = log(fabs((1.0 + eta) / (1.0 - eta)));
        const double den = 0.5 + 0.25 * (1.0 - eta * eta) / eta * A;
        ld = (0.5 / eta - 0.25 * (eta * eta + 1.0) / (eta * eta) * A) / (den * den) + 6.0 * eta * mu;
    } else if (eta < atol) {
        ld = -2.0 * eta * (1.0 / 3.0 - 3.0 * mu);
    } else if (fabs(eta - 1.0) < atol) {
        ld = -48.0;
    }
    return ld * eta;
}

template <typename T>
struct StressPointArgs {
    const T* rho;
    T* ra;  // rho^alpha (WT), or nullptr
    T* rb;  // rho^beta (WT, alpha != beta), or nullptr
    long long N;
    double alpha, beta;
    int xc;
    Consts k;
};

// rho^alpha, rho^beta as the reference's stress raises them (no clamp), the
// LDA sum of v_xc(rho) rho and the sum of rho (two float64 partials per block)
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_stress_point(StressPointArgs<T> a, double* partials) {
    using M = T;
    RunSum<M> vr, rs;
    const LdaC<M> lc(a.k);
    const M alpha = (M)a.alpha, beta = (M)a.beta;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.N; i += stride) {
        const M r = a.rho[i];
        rs.add(r);
        if (a.ra) a.ra[i] = mpow(r, alpha);
        if (a.rb) a.rb[i] = mpow(r, beta);
        if (a.xc) {
            M ex, vx;
            lda_point(r, lc, ex, vx);
            vr.add(vx * r);
        }
    }
    double acc[2] = {vr.get(), rs.get()};
    block_sum_store<2>(acc, partials);
}

__device__ __forceinline__ void sym6(double gx, double gy, double gz, double (&t)[6]) {
    t[0] = gx * gx;
    t[1] = gx * gy;
    t[2] = gx * gz;
    t[3] = gy * gy;
    t[4] = gy * gz;
    t[5] = gz * gz;
}

// Sums over the half-space mask: [0..5] g_i g_j |rho(G)|^2 / G^4 (Hartree),
// [6..11] (g_i g_j / G^2 - delta_ij / 3) L'(|G| / tkf) Re(A conj B) (WT,
// A = FFT(rho^alpha), B = FFT(rho^beta)); raw transforms.
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_stress_gspace(const typename Cplx<T>::type* __restrict__ rhoG,
                                                               const typename Cplx<T>::type* __restrict__ aG,
                                                               const typename Cplx<T>::type* __restrict__ bG, Geo geo,
                                                               double tkf, double mu, double* partials) {
    double acc[12];
    for (int k = 0; k < 12; ++k) acc[k] = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        if (!half_mask(geo, i)) continue;
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        const double inv = (i == 0) ? 0.0 : 1.0 / gg;
        double t[6];
        sym6(gx, gy, gz, t);
        if (rhoG) {
            const double rr = (double)rhoG[i].x, ri = (double)rhoG[i].y;
            const double w = (rr * rr + ri * ri) * inv * inv;
            for (int k = 0; k < 6; ++k) acc[k] += t[k] * w;
        }
        if (aG) {
            const double ar = (double)aG[i].x, ai = (double)aG[i].y;
            const double br = (double)bG[i].x, bi = (double)bG[i].y;
            const double w = lindhard_deriv_eta(sqrt(gg) / tkf, mu) * (ar * br + ai * bi);
            for (int k = 0; k < 6; ++k) {
                const double f = (k == 0 || k == 3 || k == 5) ? 1.0 / 3.0 : 0.0;
                acc[6 + k] += (t[k] * inv - f) * w;
            }
        }
    }
    block_sum_store<12>(acc, partials);
}

// sum_r d_i rho d_j rho / rho over the grid (six components)
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_stress_vw(const T* __restrict__ rho, const T* __restrict__ D,
                                                           long long N, double* partials) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const double r = (double)rho[i];
        const double dx = (double)D[i], dy = (double)D[N + i], dz = (double)D[2 * N + i];
        double t[6];
        sym6(dx, dy, dz, t);
        for (int k = 0; k < 6; ++k) acc[k] += t[k] / r;
    }
    block_sum_store<6>(acc, partials);
}

void put6(double* S, const double* v6, double scale) {
    static const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {0, 1, 2, 1, 2, 2};
    for (int k = 0; k < 6; ++k) S[3 * I[k] + J[k]] = S[3 * J[k] + I[k]] = v6[k] * scale;
}

template <typename T>
void stress_t(ofdft_eval* e, const T* rho, const double* energies, double* S, cudaStream_t st) {
    using C = typename Cplx<T>::type;
    ofdft_grid* g = e->g;
    const ofdft_config& c = e->cfg;
    OFDFT_REQUIRE(!(c.kedf_terms & OFDFT_KE_LWT), "'LWT' has not implemented.");
    double E[OFDFT_NE];
    if (energies) std::copy(energies, energies + OFDFT_NE, E);
    else compute_t<T>(e, rho, nullptr, OFDFT_CALC_E, E, st);
    // WTEStress (wte.py:25-37) evaluates the TF and WT energies itself
    const bool wte = c.wte && (c.kedf_terms & OFDFT_KE_TF) && (c.kedf_terms & OFDFT_KE_WT);
    if (wte) {
        double Er[OFDFT_NE];
        e->cfg.wte = 0;
        try {
            compute_t<T>(e, rho, nullptr, OFDFT_CALC_E, Er, st);
        } catch (...) {
            e->cfg.wte = 1;
            throw;
        }
        e->cfg.wte = 1;
        E[OFDFT_E_TF] = Er[OFDFT_E_TF];
        E[OFDFT_E_NL] = Er[OFDFT_E_NL];
    }
    for (int i = 0; i < OFDFT_NS * 9; ++i) S[i] = 0.0;
    const double V = g->volume, dV = g->dV, N = (double)g->N;
    const bool vw = c.kedf_terms & OFDFT_KE_VW, wt = c.kedf_terms & OFDFT_KE_WT;
    const bool xc = c.xc_lda != 0, h = c.hartree != 0;
    const size_t cb = g->cplx_bytes(), rb = g->real_bytes();
    const int gblk = blocks_for(g->Nc, 256, g->sms * 16);
    auto fetch = [&](int nblk, int ns) {
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, nblk, ns, 0ull, g->d_results);
        OFDFT_LAUNCH_CHECK();
        OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, ns * sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
    };
    // TF: -2/3 E/V on the diagonal
    if (c.kedf_terms & OFDFT_KE_TF)
        for (int d = 0; d < 3; ++d) S[OFDFT_S_TF * 9 + 4 * d] = -2.0 / 3.0 * E[OFDFT_E_TF] / V;
    // pointwise: rho^alpha / rho^beta, sum v_xc rho, sum rho
    const bool same_ab = c.wt_alpha == c.wt_beta;
    T* ra = wt ? (T*)e->sc.get("st_ra", rb) : nullptr;
    T* rbeta = (wt && !same_ab) ? (T*)e->sc.get("st_rb", rb) : nullptr;
    double rho0 = 0.0;
    if (wt || xc) {
        StressPointArgs<T> pa;
        pa.rho = rho;
        pa.ra = ra;
        pa.rb = rbeta;
        pa.N = g->N;
        pa.alpha = c.wt_alpha;
        pa.beta = c.wt_beta;
        pa.xc = xc ? 1 : 0;
        pa.k = e->k;
        k_stress_point<T><<<g->red_blocks, RED_THREADS, 0, st>>>(pa, g->d_partials);
        OFDFT_LAUNCH_CHECK();
        fetch(g->red_blocks, 2);
        rho0 = g->h_results[1] / N;  // rho.amean() (wt.py:77)
        if (xc) {
            const double P = E[OFDFT_E_XC] - g->h_results[0] * dV;
            for (int d = 0; d < 3; ++d) S[OFDFT_S_XC * 9 + 4 * d] = P / V;
        }
    }
    // G-space sums: Hartree and WT
    C* rhoG = (h || vw) ? (C*)e->sc.get("st_rhoG", cb) : nullptr;
    if (rhoG) g->exec_r2c(rho, rhoG, 1, st);
    C *aG = nullptr, *bG = nullptr;
    double tkf = 1.0;
    if (wt) {
        aG = (C*)e->sc.get("st_aG", cb);
        g->exec_r2c(ra, aG, 1, st);
        bG = aG;
        if (!same_ab) {
            bG = (C*)e->sc.get("st_bG", cb);
            g->exec_r2c(rbeta, bG, 1, st);
        }
        tkf = 2.0 * std::pow(3.0 * rho0 * M_PI * M_PI, 1.0 / 3.0);  // wt.py:86
    }
    if (h || wt) {
        k_stress_gspace<T><<<g->red_blocks, RED_THREADS, 0, st>>>(h ? rhoG : nullptr, aG, bG, g->geo, tkf, c.vw_y,
                                                                   g->d_partials);
        OFDFT_LAUNCH_CHECK();
        fetch(g->red_blocks, 12);
        const double* R = g->h_results;
        if (h) {
            // 8 pi / V^2 sum |rho_ref|^2 g_i g_j / G^4 with rho_ref = dV FFT(rho); -E_H/V on the diagonal
            put6(S + OFDFT_S_H * 9, R, 8.0 * M_PI / (V * V) * dV * dV);
            for (int d = 0; d < 3; ++d) S[OFDFT_S_H * 9 + 4 * d] -= E[OFDFT_E_H] / V;
        }
        if (wt) {
            // DDrho = L' A_ref conj(B_ref) / V^2 = L' A conj(B) / N^2 (raw transforms), times
            // pi^2 / (alpha beta rho0^(alpha+beta-2) tkf/2); -2/3 E_WT/V on the diagonal (wt.py:86-106)
            const double pre = M_PI * M_PI /
                               (c.wt_alpha * c.wt_beta * std::pow(rho0, c.wt_alpha + c.wt_beta - 2.0) * tkf / 2.0);
            put6(S + OFDFT_S_NL * 9, R + 6, pre / (N * N));
            for (int d = 0; d < 3; ++d) S[OFDFT_S_NL * 9 + 4 * d] -= 2.0 / 3.0 * E[OFDFT_E_NL] / V;
        }
    }
    // GGA (gga.py:1306-1318): P = E - int pot1 rho - sum_i int w (d_i rho)^2, sigma_ii = P - int w (d_i rho)^2,
    // sigma_ij = -int w d_i rho d_j rho, w = tf F' / rho^(8/3), over V
    if (c.kedf_terms & OFDFT_KE_GGA) {
        OFDFT_REQUIRE(c.gga_formula < OFDFT_GGA_GE2, "ofdft_eval_stress: no stress for a meta-GGA (gga.py:1313-1314)");
        gga_enqueue<T>(g, e->sc, gga_spec(c), rho, nullptr, false, true, g->d_results + 40, st);
        OFDFT_CK(cudaMemcpyAsync(g->h_results + 40, g->d_results + 40, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        const double* R = g->h_results + 40;
        const double P = R[0] * dV - R[1] * dV - (R[2] + R[5] + R[7]) * dV;
        double w6[6];
        for (int k = 0; k < 6; ++k) w6[k] = -R[2 + k] * dV / V;
        put6(S + OFDFT_S_GGA * 9, w6, 1.0);
        for (int d = 0; d < 3; ++d) S[OFDFT_S_GGA * 9 + 4 * d] += P / V;
    }
    // vW: -(y/4) dV/V sum d_i rho d_j rho / rho
    if (vw) {
        C* X = (C*)e->sc.get("st_X", 3 * cb);
        T* D = (T*)e->sc.get("st_D", 3 * rb);
        k_grad_spectra<T><<<gblk, 256, 0, st>>>(rhoG, X, g->geo, 1.0 / N, 0.0, 0);
        OFDFT_LAUNCH_CHECK();
        g->exec_c2r(X, D, 3, st);
        k_stress_vw<T><<<g->red_blocks, RED_THREADS, 0, st>>>(rho, D, g->N, g->d_partials);
        OFDFT_LAUNCH_CHECK();
        fetch(g->red_blocks, 6);
        put6(S + OFDFT_S_VW * 9, g->h_results, -0.25 / V * dV * c.vw_y);
    }
    // WTE (wte.py:33-37): exp(E_WT/E_TF) (sigma_WT + 2/3 E_WT/V on the diagonal + sigma_TF), in the NL slot
    if (wte) {
        const double ex = std::exp(E[OFDFT_E_NL] / E[OFDFT_E_TF]);
        for (int d = 0; d < 3; ++d) S[OFDFT_S_NL * 9 + 4 * d] += 2.0 / 3.0 * E[OFDFT_E_NL] / V;
        for (int k = 0; k < 9; ++k) {
            S[OFDFT_S_NL * 9 + k] = (S[OFDFT_S_NL * 9 + k] + S[OFDFT_S_TF * 9 + k]) * ex;
            S[OFDFT_S_TF * 9 + k] = 0.0;
        }
    }
}

}  // namespace

extern "C" {

size_t ofdft_config_size(void) { return sizeof(ofdft_config); }

void ofdft_config_default(ofdft_config* c) {
    memset(c, 0, sizeof(*c));
    c->struct_size = (unsigned)sizeof(ofdft_config);
    c->kedf_terms = OFDFT_KE_TF | OFDFT_KE_VW;
    c->tf_x = 1.0;
    c->vw_y = 1.0;
    c->wt_alpha = c->wt_beta = 5.0 / 6.0;
    c->wt_x = 1.0;
    c->wt_rho0 = 0.0;
    c->lwt_alpha = c->lwt_beta = 5.0 / 6.0;
    c->lwt_x = 1.0;
    c->lwt_nsp = 0;
    c->lwt_delta = 0.0;
    c->lwt_ratio = 1.15;
    c->lwt_kdd = 3;
    c->lwt_interp = OFDFT_INTERP_LINEAR;
    c->lwt_etamax = 50.0;
    c->lwt_neta = 50000;
    c->lwt_kfmin = NAN;
    c->lwt_kfmax = NAN;
    c->lwt_ldw = 1.0 / 6.0;
    c->lwt_max_batch = 0;
    c->lwt_kernel = OFDFT_LWT_KERNEL_WT;
    c->lwt_maxpoints = 1000;
    c->gga_formula = OFDFT_GGA_LKT;  // GGA_KEDF_list["LKT"] (gga.py:589)
    c->gga_nparams = 2;
    c->gga_params[0] = 1.3;
    c->gga_params[1] = 1.0;
    c->gga_remove_vw = 0.0;
    c->lwt_family = OFDFT_LWT_FAMILY_LWT;
    c->wt_kernel = OFDFT_LWT_KERNEL_WT;
    c->wt_maxpoints = 1000;
    c->wt_lump = 0;
    c->wt_lump_abc[0] = 0.2;
    c->wt_lump_abc[1] = 0.2;
    c->wt_lump_abc[2] = 1.0;
    c->wt_revke = 1;
    c->xc_lda = 1;
    c->hartree = 1;
    c->pseudo = 0;
    c->ewald_energy = 0.0;
}

int ofdft_config_init(ofdft_config* c, size_t caller_size) {
    return guard([&] {
        OFDFT_REQUIRE(c, "ofdft_config_init: null argument");
        OFDFT_REQUIRE(caller_size == sizeof(ofdft_config),
                      "ofdft_config_init: the caller's struct has %zu bytes, this library's ofdft_config %zu: "
                      "rebuild the binding from include/ofdft.h",
                      caller_size, sizeof(ofdft_config));
        ofdft_config_default(c);
    });
}

int ofdft_eval_create(ofdft_grid* g, const ofdft_config* cfg, ofdft_eval** out) {
    return guard([&] {
        OFDFT_REQUIRE(cfg && out, "ofdft_eval_create: null argument");
        OFDFT_REQUIRE(cfg->struct_size == sizeof(ofdft_config),
                      "ofdft_eval_create: ofdft_config.struct_size = %u, this library's ofdft_config has %zu bytes: "
                      "fill the config with ofdft_config_init, from a binding that mirrors include/ofdft.h",
                      cfg->struct_size, sizeof(ofdft_config));
        OFDFT_REQUIRE(g, "ofdft_eval_create: null grid");
        const ofdft_config& c = *cfg;
        OFDFT_REQUIRE(!((c.kedf_terms & OFDFT_KE_WT) && (c.kedf_terms & OFDFT_KE_LWT)),
                      "only one nonlocal KEDF term at a time");
        if (c.kedf_terms & OFDFT_KE_GGA) {
            OFDFT_REQUIRE(c.gga_formula >= 0 && c.gga_formula < OFDFT_GGA_NFORMULAS, "gga_formula out of range");
            OFDFT_REQUIRE(c.gga_nparams >= 1 && c.gga_nparams <= 8, "gga_nparams must be 1..8");
        }
        if (c.kedf_terms & OFDFT_KE_LWT) {
            OFDFT_REQUIRE(c.lwt_kdd >= 1 && c.lwt_kdd <= 3, "lwt_kdd must be 1, 2 or 3");
            OFDFT_REQUIRE(c.lwt_neta >= 4 && c.lwt_etamax > 0, "bad kernel table size");
            OFDFT_REQUIRE(c.lwt_interp == OFDFT_INTERP_LINEAR || c.lwt_interp == OFDFT_INTERP_HERMITE,
                          "lwt_interp must be linear or hermite");
            OFDFT_REQUIRE(c.lwt_nsp > 0 || c.lwt_delta > 0 || c.lwt_ratio > 1.0, "need nsp, delta or ratio > 1");
            OFDFT_REQUIRE(c.lwt_nsp != 1, "nsp must be >= 2");
            OFDFT_REQUIRE(c.lwt_kernel >= OFDFT_LWT_KERNEL_WT && c.lwt_kernel <= OFDFT_LWT_KERNEL_USER,
                          "lwt_kernel must be one of OFDFT_LWT_KERNEL_*");
            OFDFT_REQUIRE(c.lwt_family == OFDFT_LWT_FAMILY_LWT || c.lwt_family == OFDFT_LWT_FAMILY_HC,
                          "lwt_family must be one of OFDFT_LWT_FAMILY_*");
            OFDFT_REQUIRE(c.lwt_family != OFDFT_LWT_FAMILY_HC ||
                              (c.lwt_interp == OFDFT_INTERP_HERMITE && c.gga_formula >= 0 &&
                               c.gga_formula < OFDFT_GGA_GE2 && c.gga_nparams >= 1 && c.gga_nparams <= 8),
                          "HC: Hermite interpolation and a GGA enhancement factor are required");
            OFDFT_REQUIRE(c.lwt_kernel == OFDFT_LWT_KERNEL_WT || c.lwt_maxpoints >= 1, "lwt_maxpoints must be >= 1");
        }
        if (c.kedf_terms & OFDFT_KE_WT) {
            OFDFT_REQUIRE(c.wt_kernel >= OFDFT_LWT_KERNEL_WT && c.wt_kernel <= OFDFT_LWT_KERNEL_MGPG,
                          "wt_kernel must be OFDFT_LWT_KERNEL_WT, _MGP, _MGPA or _MGPG");
            OFDFT_REQUIRE(c.wt_kernel == OFDFT_LWT_KERNEL_WT || (c.wt_maxpoints >= 1 && !c.wte),
                          "MGP kernels: wt_maxpoints >= 1, and not with WTE");
            OFDFT_REQUIRE(c.wt_lump >= 0 && c.wt_lump <= 2, "wt_lump must be 0, 1 or 2");
        }
        auto* e = new ofdft_eval();
        e->g = g;
        e->cfg = c;
        e->k = make_consts();
        try {
            OFDFT_CK(cudaMalloc(&e->wtstate, 8 * sizeof(double)));
            zero_now(e->wtstate, 8 * sizeof(double));
            if ((c.kedf_terms & OFDFT_KE_WT) && c.wt_kernel != OFDFT_LWT_KERNEL_WT) {
                // MGPKernelTable (kernel.py:281-292): splrep of LindhardFunction(eta, 1, 1) on
                // logspace(log10(1e-4), log10(52), 10000)
                const int n = 10000;
                const double l0 = std::log10(1e-4), l1 = std::log10(52.0), step = (l1 - l0) / (n - 1);
                std::vector<double> x(n), y(n);
                for (int i = 0; i < n; ++i) {
                    x[i] = std::pow(10.0, i == n - 1 ? l1 : l0 + i * step);
                    y[i] = lindhard(x[i], 1.0, 1.0);
                }
                CubicSpline sp;
                sp.fit(x, y);
                e->mgp_n = n;
                OFDFT_CK(cudaMalloc(&e->mgp_x, n * sizeof(double)));
                OFDFT_CK(cudaMalloc(&e->mgp_c, sp.c.size() * sizeof(double)));
                upload_now(e->mgp_x, sp.x.data(), n * sizeof(double));
                upload_now(e->mgp_c, sp.c.data(), sp.c.size() * sizeof(double));
            }
            if (c.kedf_terms & OFDFT_KE_LWT) {
                if (g->prec == OFDFT_F64) build_table<double>(e);
                else build_table<float>(e);
                OFDFT_CK(cudaMalloc(&e->d_nodes, 3 * kMaxNodes * sizeof(double)));
                OFDFT_CK(cudaMallocHost(&e->h_nodes, 3 * kMaxNodes * sizeof(double)));
            }
        } catch (...) {
            ofdft_eval_destroy(e);
            throw;
        }
        *out = e;
    });
}

void ofdft_eval_destroy(ofdft_eval* e) {
    if (!e) return;
    e->sc.release_all();
    if (e->vloc) cudaFree(e->vloc);
    if (e->vext) cudaFree(e->vext);
    if (e->mgp_x) cudaFree(e->mgp_x);
    if (e->mgp_c) cudaFree(e->mgp_c);
    if (e->wtstate) cudaFree(e->wtstate);
    if (e->tab_c) cudaFree(e->tab_c);
    if (e->tab_cd) cudaFree(e->tab_cd);
    if (e->d_nodes) cudaFree(e->d_nodes);
    if (e->h_nodes) cudaFreeHost(e->h_nodes);
    if (e->fz_tw) cudaFree(e->fz_tw);
    if (e->fz_st2) cudaStreamDestroy(e->fz_st2);
    if (e->fz_fork) cudaEventDestroy(e->fz_fork);
    if (e->fz_join) cudaEventDestroy(e->fz_join);
    if (e->d_fz_err) cudaFree(e->d_fz_err);
    if (e->h_fz_err) cudaFreeHost(e->h_fz_err);
    for (auto ev : e->evs) cudaEventDestroy(ev);
    delete e;
}

int ofdft_eval_set_vloc(ofdft_eval* e, const void* vloc_dev, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(e && vloc_dev, "ofdft_eval_set_vloc: null argument");
        if (!e->vloc) OFDFT_CK(cudaMalloc(&e->vloc, e->g->real_bytes()));
        OFDFT_CK(cudaMemcpyAsync(e->vloc, vloc_dev, e->g->real_bytes(), cudaMemcpyDeviceToDevice, (cudaStream_t)s));
        e->have_vloc = true;
    });
}

int ofdft_eval_set_external(ofdft_eval* e, const void* v_dev, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(e && v_dev, "ofdft_eval_set_external: null argument");
        if (!e->vext) OFDFT_CK(cudaMalloc(&e->vext, e->g->real_bytes()));
        OFDFT_CK(cudaMemcpyAsync(e->vext, v_dev, e->g->real_bytes(), cudaMemcpyDeviceToDevice, (cudaStream_t)s));
        e->have_vext = true;
    });
}

int ofdft_eval_set_ewald(ofdft_eval* e, double energy) {
    return guard([&] {
        OFDFT_REQUIRE(e, "ofdft_eval_set_ewald: null evaluator");
        e->cfg.ewald_energy = energy;
    });
}

int ofdft_eval_compute(ofdft_eval* e, const void* rho, void* v_out, unsigned calc, double* energies, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(e && rho && energies, "ofdft_eval_compute: null argument");
        OFDFT_REQUIRE(calc & (OFDFT_CALC_E | OFDFT_CALC_V), "ofdft_eval_compute: calc must include E or V");
        if (e->g->prec == OFDFT_F64)
            compute_t<double>(e, (const double*)rho, (double*)v_out, calc, energies, (cudaStream_t)s);
        else
            compute_t<float>(e, (const float*)rho, (float*)v_out, calc, energies, (cudaStream_t)s);
    });
}

int ofdft_eval_stress(ofdft_eval* e, const void* rho, const double* energies, double* stress, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(e && rho && stress, "ofdft_eval_stress: null argument");
        if (e->g->prec == OFDFT_F64) stress_t<double>(e, (const double*)rho, energies, stress, (cudaStream_t)s);
        else stress_t<float>(e, (const float*)rho, energies, stress, (cudaStream_t)s);
    });
}

int ofdft_eval_set_lwt_table(ofdft_eval* e, const double* table, int neta) {
    return guard([&] {
        OFDFT_REQUIRE(e && table, "ofdft_eval_set_lwt_table: null argument");
        OFDFT_REQUIRE(e->cfg.kedf_terms & OFDFT_KE_LWT, "ofdft_eval_set_lwt_table: no k_F-node term configured");
        OFDFT_REQUIRE(neta == e->cfg.lwt_neta, "ofdft_eval_set_lwt_table: %d values, the evaluator has lwt_neta %d",
                      neta, e->cfg.lwt_neta);
        const std::vector<double> eta = table_eta(e->cfg);
        const std::vector<double> y(table, table + neta);
        if (e->g->prec == OFDFT_F64) upload_table<double>(e, eta, y);
        else upload_table<float>(e, eta, y);
    });
}

int ofdft_eval_get_kfbounds(const ofdft_eval* e, double* kfmin, double* kfmax) {
    return guard([&] {
        OFDFT_REQUIRE(e && kfmin && kfmax, "ofdft_eval_get_kfbounds: null argument");
        *kfmin = e->kf_set_min ? e->kf_st_min : NAN;
        *kfmax = e->kf_set_max ? e->kf_st_max : NAN;
    });
}

int ofdft_eval_set_kfbounds(ofdft_eval* e, double kfmin, double kfmax) {
    return guard([&] {
        OFDFT_REQUIRE(e, "ofdft_eval_set_kfbounds: null evaluator");
        e->kf_set_min = !std::isnan(kfmin);
        e->kf_st_min = kfmin;
        e->kf_set_max = !std::isnan(kfmax);
        e->kf_st_max = kfmax;
    });
}

int ofdft_eval_profile(ofdft_eval* e, int enable) {
    return guard([&] {
        OFDFT_REQUIRE(e, "ofdft_eval_profile: null evaluator");
        e->prof = enable != 0;
        for (int i = 0; i < ofdft_eval::kClasses; ++i) {
            e->prof_ms[i] = 0.0;
            e->prof_bytes[i] = 0.0;
            e->prof_launches[i] = 0;
        }
        e->rec_cls.clear();
        e->rec_bytes.clear();
    });
}

int ofdft_eval_profile_read(const ofdft_eval* e, int max_classes, double* ms, double* bytes, long long* launches,
                            int* nclasses) {
    return guard([&] {
        OFDFT_REQUIRE(e && nclasses, "ofdft_eval_profile_read: null argument");
        const int n = std::min(max_classes, (int)ofdft_eval::kClasses);
        for (int i = 0; i < n; ++i) {
            if (ms) ms[i] = e->prof_ms[i];
            if (bytes) bytes[i] = e->prof_bytes[i];
            if (launches) launches[i] = e->prof_launches[i];
        }
        *nclasses = ofdft_eval::kClasses;
    });
}

const char* ofdft_profile_class_name(int i) {
    return (i >= 0 && i < ofdft_eval::kClasses) ? kProfNames[i] : nullptr;
}

int ofdft_eval_last_stats(const ofdft_eval* e, int* nsp, int* launches) {
    return guard([&] {
        OFDFT_REQUIRE(e, "ofdft_eval_last_stats: null evaluator");
        if (nsp) *nsp = e->last_nsp;
        if (launches) *launches = e->last_launches;
    });
}

}  // extern "C"
