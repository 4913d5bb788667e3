// Fused float32 pipeline of the density-dependent (k_F-node) kernel for
// power-of-two grids (each axis 32..256, the contiguous axis 32..512).
//
// It computes what the cuFFT pipeline computes (lwt.py:226-306, kernel.py:379-405):
//   P_j = IFFT(K_j FFT(rho^beta)/N), M_j = IFFT(K'_j/k_j FFT(rho^beta)/N)
//   pot1 (+)= linear interpolation of P over each point's k_F interval
//   pot3 (+)= the same interpolation of M                          (kdd = 3)
//   pot2(G) (+)= sum_j K_j(G) FFT(rho^alpha W_j)(G)/N              (kdd > 1)
// or, with the cubic Hermite interpolation, pot1 and pot3 from both P and M
// and pot2(G) (+)= sum_j K_j FFT(rho^alpha W_j)/N + K'_j/k_j FFT(rho^alpha WD_j)/N
// with the Hermite basis weights W_j, WD_j (fz_hermite_w)
// with the node kernel, the interpolation and the hat weights folded into
// hand-written tile FFTs, so the node planes cross HBM three times each
// instead of five and no real-space plane is stored:
//   C2R: k_fz_nodes    axis 0 inverse, K_j and K'_j applied on load
//        k_fz_axis1    axis 1 inverse
//        k_fz_c2r_rows axis 2 C2R, interpolated into pot1/pot3 per point
//   R2C: k_fz_r2c_rows hat weights times rho^alpha, axis 2 R2C
//        k_fz_axis1    axis 1 forward
//        k_fz_pot2     axis 0 forward, K_j applied and summed into pot2(G)
// Intermediate planes hold k2 < n2/2 as [n0][n1][n2/2] followed by the
// Nyquist column k2 = n2/2 as [n0][n1]; pot2(G) and FFT(rho^beta) use the
// R2C half-grid layout [n0][n1][n2/2+1].
//
// Nothing in these kernels runs on the float64 pipe inside a node loop: the
// kernel-table parameters come in float32 (FzTab), and the interval
// membership of each point is decided in float32 against node bounds rounded
// outward (__double2float_rd/_ru), which reproduces the float64 comparisons of
// the reference exactly for float32 k_F values.
#pragma once
#include "fz_fft.cuh"

namespace {

struct FzDims {
    int n0, n1, n2, H;  // H = n2/2
    long long nyq;      // n0*n1*H: offset of the Nyquist block in a plane
    long long plane;    // n0*n1*(H+1) complex per plane
};

struct FzTw {
    const float2* t0;  // exp(-2 pi i k/n0), k < n0
    const float2* t1;  // exp(-2 pi i k/n1), k < n1
    const float2* th;  // exp(-2 pi i k/H),  k < H
    const float2* tr;  // exp(-2 pi i k/n2), k < H
    const float2* tq;  // exp(-2 pi i k/32), k < 32 (split path)
};

constexpr int kFzLines = 16;  // lines per column tile
constexpr int kFzColE = 16;   // points per thread along a column
constexpr int kFzRowE = 8;    // complex points per thread along a row
constexpr int kFzRowThreads = 256;

// float32 copy of the kernel-table parameters
struct FzTab {
    const float* c;   // K(eta) cubic pieces
    const float* cd;  // -eta K'(eta) cubic pieces
    int nint;
    float step, inv_step, etamax, limit, limitd, factor, kconst, eta_series;  // kconst = -lbda - 0.6
};

FzTab fz_tab(const Table<float>& t) {
    FzTab f;
    f.c = t.c;
    f.cd = t.cd;
    f.nint = t.nint;
    f.step = (float)t.step;
    f.inv_step = (float)t.inv_step;
    f.etamax = (float)t.etamax;
    f.limit = (float)t.limit;
    f.limitd = (float)t.limitd;
    f.factor = (float)t.factor;
    f.kconst = (float)(-t.lbda - 0.6);
    // spline below eta_series; never at or above etamax, where the table limit applies
    f.eta_series = (float)std::min(t.eta_series, t.etamax);
    return f;
}

// Coefficients c_k of the large-eta series of the inverse Lindhard function
// with mu = 1 (kernel.py:79-133): F = -lbda - 0.6 + sum_k c_k eta^{-2(k+1)}.
// For eta >= 2.5 the terms after k = 7 are below 5e-10 of F, and those of
// -eta F' after k = 9 below 1e-8 of it, so eight terms (ten for the
// derivative) reproduce the table to float32 precision.
__device__ __forceinline__ constexpr float fz_series_c(int k) {
    return k == 0   ? -0.13714285714285712f
           : k == 1 ? -6.39999999999999875e-2f
           : k == 2 ? -3.77825602968460128e-2f
           : k == 3 ? -2.51824061652633074e-2f
           : k == 4 ? -1.80879839616166146e-2f
           : k == 5 ? -1.36715733124818332e-2f
           : k == 6 ? -1.07236045520990083e-2f
           : k == 7 ? -8.65192783339199453e-3f
           : k == 8 ? -7.1372762502456763e-3f
                    : -5.9945117538835746e-3f;
}

__device__ __forceinline__ float fz_spline(const float* c, int nint, float step, float inv_step, float eta) {
    int l = (int)(eta * inv_step);
    l = l < 0 ? 0 : (l >= nint ? nint - 1 : l);
    const float u = eta - (float)l * step;
    const float4 q = __ldg(reinterpret_cast<const float4*>(c) + l);
    return q.x + u * (q.y + u * (q.z + u * q.w));
}

// K_j(|G|) (DERIV false) or -eta K_j'(eta) (DERIV true) at eta = q/k_j: the
// table limit at and above etamax, the series at and above eta_series
// (u = eta^-2 = k_j^2/q^2), the spline below (NEAR only: callers pass
// NEAR = false when no point of the warp can have eta < eta_series, so that
// warp runs no spline instructions at all).  G = 0 is handled by the callers.
template <bool DERIV, bool NEAR>
__device__ __forceinline__ float fz_node_kernel(const FzTab& tb, float q, float ik, float iq2, float kj2) {
    const float eta = q * ik;
    const float u = iq2 * kj2;
    float r;
    if constexpr (DERIV) {
        float d = 20.0f * fz_series_c(9);
#pragma unroll
        for (int k = 8; k >= 0; --k) d = fmaf(d, u, (float)(2 * (k + 1)) * fz_series_c(k));
        r = tb.factor * (d * u);
        r = eta >= tb.etamax ? tb.limitd : r;
    } else {
        float f = fz_series_c(7);
#pragma unroll
        for (int k = 6; k >= 0; --k) f = fmaf(f, u, fz_series_c(k));
        r = tb.factor * fmaf(f, u, tb.kconst);
        r = eta >= tb.etamax ? tb.limit : r;
    }
    if constexpr (NEAR) {
        if (eta < tb.eta_series) r = fz_spline(DERIV ? tb.cd : tb.c, tb.nint, tb.step, tb.inv_step, eta);
    }
    return r;
}

// Smallest |G| over the 32 lanes' points (|G| >= 0, so its bits order as unsigned).
__device__ __forceinline__ float fz_warp_min(float x) {
    return __uint_as_float(__reduce_min_sync(0xffffffffu, __float_as_uint(x)));
}

// Column tile of the axis-0 passes: main tiles (k1, 16 consecutive k2 < H) then
// Nyquist tiles (16 consecutive k1, k2 = H).  Sets k1, k2 of this thread's line,
// the offset/stride in a plane and the offset/stride in the half-grid layout.
__device__ __forceinline__ void fz_axis0_tile(const FzDims& d, int tile, int l, int& k1, int& k2, long long& pbase,
                                              long long& pstride, long long& gbase, long long& gstride) {
    const int per_row = d.H / kFzLines;
    const int tiles_main = d.n1 * per_row;
    if (tile < tiles_main) {
        k1 = tile / per_row;
        k2 = (tile % per_row) * kFzLines + l;
        pbase = (long long)k1 * d.H + k2;
        pstride = (long long)d.n1 * d.H;
    } else {
        k1 = (tile - tiles_main) * kFzLines + l;
        k2 = d.H;
        pbase = d.nyq + k1;
        pstride = d.n1;
    }
    gbase = (long long)k1 * (d.H + 1) + k2;
    gstride = (long long)d.n1 * (d.H + 1);
}

// Shared-memory size of k_fz_nodes / k_fz_pot2 for column length n0 and nb nodes.
inline size_t fz_col_smem(int n0, int nb, bool with_b) {
    const size_t pts = (size_t)n0 * kFzLines;
    return fz::col_slots(n0) * sizeof(float2) + pts * (2 * sizeof(float) + (with_b ? sizeof(float2) : 0)) +
           2 * (size_t)nb * sizeof(float);
}

// X_j = K_j FFT(rho^beta)/N (DERIV false) or Y_j = K'_j/k_j FFT(rho^beta)/N
// (DERIV true) of the block's share of a batch of nodes, inverse-transformed
// along axis 0 into plane `plane0 + jj`.  Block b handles tile b % tiles and
// node share b / tiles of nsplit.  The tile's FFT(rho^beta)/N, |G| and 1/|G|^2
// sit in shared memory for the whole node loop; FFT(rho^beta) at G = 0 is
// zeroed there, which is K_j(0) = 0.
template <int N0, bool DERIV>
__global__ void __launch_bounds__(kFzLines * (N0 / kFzColE), 2)
    k_fz_nodes(const float2* __restrict__ rbG, float2* __restrict__ XY, FzTab tb, const double* __restrict__ knode,
               const double* __restrict__ invk, int j0, int nb, int plane0, int tiles, int nsplit, Geo geo,
               FzDims d, const float2* __restrict__ tw, float invN) {
    constexpr int E = kFzColE, T = N0 / E, L = kFzLines;
    extern __shared__ float2 fz_sm[];
    float2* sm = fz_sm;
    float2* sz = fz_sm + fz::col_slots(N0);
    float* sq = reinterpret_cast<float*>(sz + N0 * L);
    float* siq = sq + N0 * L;
    float* sik = siq + N0 * L;
    float* sk2 = sik + nb;
    const int tile = blockIdx.x % tiles, part = blockIdx.x / tiles;
    const int per = (nb + nsplit - 1) / nsplit;
    const int s0 = part * per, s1 = min(nb, s0 + per);
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        const double k = knode[j0 + q];
        sik[q] = (float)invk[j0 + q];
        sk2[q] = (float)(k * k);
    }
    const int l = threadIdx.x % L, t = threadIdx.x / L;
    int k1, k2;
    long long pbase, pstride, gbase, gstride;
    fz_axis0_tile(d, tile, l, k1, k2, pbase, pstride, gbase, gstride);
#pragma unroll 4
    for (int e = 0; e < E; ++e) {
        const int k0 = t + T * e;
        const int s = k0 * L + l;
        float2 a = __ldg(rbG + gbase + k0 * gstride);
        a = make_float2(a.x * invN, a.y * invN);
        const float q2 = gsq_f(geo, k0, k1, k2);
        if (k0 == 0 && k1 == 0 && k2 == 0) a = make_float2(0.0f, 0.0f);
        sz[s] = a;
        sq[s] = sqrtf(q2);
        siq[s] = q2 > 0.0f ? 1.0f / q2 : 0.0f;
    }
    float2 twr[fz::tw_count<N0, E>()];
    fz::tw_load<N0, E>(twr, t, tw);
    __syncthreads();
    float qmin = INFINITY;
#pragma unroll
    for (int e = 0; e < E; ++e) qmin = fminf(qmin, sq[(t + T * e) * L + l]);
    qmin = fz_warp_min(qmin);
    for (int jj = s0; jj < s1; ++jj) {
        const float ik = sik[jj], kj2 = sk2[jj];
        float2 v[E];
        auto scale = [&](auto near) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int s = (t + T * e) * L + l;
                const float kv = fz_node_kernel<DERIV, decltype(near)::value>(tb, sq[s], ik, siq[s], kj2);
                const float f = DERIV ? kv * ik : kv;
                const float2 z = sz[s];
                v[e] = make_float2(f * z.x, f * z.y);
            }
        };
        // warp-uniform: does any point of this warp need the spline for node j?
        if (qmin * ik < tb.eta_series) scale(std::true_type());
        else scale(std::false_type());
        __syncthreads();  // the exchange buffer is free
        fz::line_fft_r<N0, E, +1>(v, sm + l, fz::ColIdx(), t, twr);
        float2* outp = XY + (long long)(plane0 + jj) * d.plane + pbase + t * pstride;
        const long long step = (long long)T * pstride;
#pragma unroll
        for (int e = 0; e < E; ++e) __stcs(outp + e * step, v[e]);
    }
}

// Axis-1 transform of every plane, in place.  Main tiles: (i0, 16 consecutive
// k2) with lines across threads; Nyquist tiles: 16 consecutive i0, whose lines
// are contiguous, with the points of a line across threads.
template <int N1, int S>
__global__ void __launch_bounds__(kFzLines * (N1 / kFzColE))
    k_fz_axis1(float2* __restrict__ XY, FzDims d, const float2* __restrict__ tw) {
    constexpr int E = kFzColE, T = N1 / E;
    extern __shared__ float2 fz_sm[];
    const int per_row = d.H / kFzLines;
    const int tiles_main = d.n0 * per_row;
    const int tiles = tiles_main + d.n0 / kFzLines;
    const int p = blockIdx.x / tiles, tile = blockIdx.x % tiles;
    float2* base = XY + (long long)p * d.plane;
    float2 v[E];
    if (tile < tiles_main) {
        const int l = threadIdx.x % kFzLines, t = threadIdx.x / kFzLines;
        const int i0 = tile / per_row, k2 = (tile % per_row) * kFzLines + l;
        float2* line = base + (long long)i0 * N1 * d.H + k2;
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = __ldcs(line + (long long)(t + T * e) * d.H);
        fz::line_fft<N1, E, S>(v, fz_sm + l, fz::ColIdx(), t, tw);
#pragma unroll
        for (int e = 0; e < E; ++e) __stcs(line + (long long)(t + T * e) * d.H, v[e]);
    } else {
        const int t = threadIdx.x % T, l = threadIdx.x / T;
        const int i0 = (tile - tiles_main) * kFzLines + l;
        float2* line = base + d.nyq + (long long)i0 * N1;
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = __ldcs(line + t + T * e);
        fz::line_fft<N1, E, S>(v, fz_sm + l * fz::row_slots(N1), fz::RowIdx(), t, tw);
#pragma unroll
        for (int e = 0; e < E; ++e) __stcs(line + t + T * e, v[e]);
    }
}

struct FzRowArgs {
    const float* kf;
    const float* rA;
    float2* XY;
    float* pot1;
    float* pot3;
    const double* kn;
    const double* kup;
    int m, j0, nb, first;
    double kfclip;
    FzDims d;
    FzTw tw;
    unsigned* err;  // set to 1 when a copy into shared memory did not complete in time
};

// Node bounds of the interval search in float32, staged per block (6 m floats):
//   kdn  = kn rounded down:  kn < kf  <=> kdn < kf,  kf <= kn <=> kf <= kdn
//   kupu = kup rounded up:   kf < kup <=> kf < kupu
//   khi + klo = kn (two floats), iw = 1/(kn[i+1] - kn[i]), dk = kn[i+1] - kn[i]
// for float32 kf.  iw[m-1] holds 1/kn[0] (the small-k_F coordinate), dk[m-1] 0.
struct FzNodeSm {
    const float *kdn, *kupu, *khi, *klo, *iw, *dk;
};

__device__ __forceinline__ FzNodeSm fz_stage_nodes(const FzRowArgs& a, float* s) {
    const int m = a.m;
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
        const double k = a.kn[q];
        const float hi = __double2float_rn(k);
        s[q] = __double2float_rd(k);
        s[m + q] = __double2float_ru(a.kup[q]);
        s[2 * m + q] = hi;
        s[3 * m + q] = __double2float_rn(k - (double)hi);
        s[4 * m + q] = __double2float_rn(q + 1 < m ? 1.0 / (a.kn[q + 1] - k) : 1.0 / a.kn[0]);
        s[5 * m + q] = q + 1 < m ? __double2float_rn(a.kn[q + 1] - k) : 0.0f;
    }
    FzNodeSm n;
    n.kdn = s;
    n.kupu = s + m;
    n.khi = s + 2 * m;
    n.klo = s + 3 * m;
    n.iw = s + 4 * m;
    n.dk = s + 5 * m;
    return n;
}

// Cubic Hermite weights of node j at a point of interval coordinate t whose
// interval starts at j (lo) or ends at j (hi), as the reference forms them
// (lwt.py:275-306, h00 = 2t^3 - 3t^2 + 1, h01 = 1 - h00, h10 = t^3 - 2t^2 + t,
// h11 = t^3 - t^2 and their t-derivatives): for the P planes w1 = h00 | h01 and
// w3 = h00' / D0 | h01' / D1; for the M planes w1 = D0 h10 | D1 h11 and
// w3 = h10' | h11'; D0 = k_{j+1} - k_j, D1 = k_j - k_{j-1}; zero elsewhere.
template <bool MPLANE>
__device__ __forceinline__ void fz_hermite_w(float t, bool lo, bool hi, float D0, float D1, float iD0, float iD1,
                                             float& w1, float& w3) {
    if constexpr (!MPLANE) {
        const float h00 = fmaf(t * t, fmaf(2.0f, t, -3.0f), 1.0f);
        const float hd = 6.0f * t * (t - 1.0f);  // h00'; h01' = -h00'
        w1 = lo ? h00 : (hi ? 1.0f - h00 : 0.0f);
        w3 = lo ? hd * iD0 : (hi ? -hd * iD1 : 0.0f);
    } else {
        const float u = t * (t - 1.0f);
        w1 = lo ? D0 * (u * (t - 1.0f)) : (hi ? D1 * (u * t) : 0.0f);
        w3 = lo ? (3.0f * t - 1.0f) * (t - 1.0f) : (hi ? t * (3.0f * t - 2.0f) : 0.0f);
    }
}

// Interval membership of the reference (lwt.py:252-306) in float32 with the
// closed-interior rule of the float32 path (a point exactly on an interior node
// joins the interval below it): il = containing interval or -1, small = the
// small-k_F branch of node 0, with their coordinates.  At most one interval
// contains a point under this rule.
__device__ __forceinline__ void fz_member(float kf, const FzNodeSm& n, int m, int& il, float& til, bool& small,
                                          float& tsm) {
    int lo = 0, hi = m;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (n.kdn[mid] < kf) lo = mid + 1;
        else hi = mid;
    }
    const int i1 = lo - 1, i2 = lo - 2;
    auto below_top = [&](int i) { return (i + 1 <= m - 2) ? kf <= n.kdn[i + 1] : kf < n.kupu[i + 1]; };
    const bool in1 = i1 >= 0 && i1 <= m - 2 && below_top(i1);
    const bool in2 = i2 >= 0 && i2 <= m - 2 && below_top(i2);
    il = in1 ? i1 : (in2 ? i2 : -1);
    til = il >= 0 ? ((kf - n.khi[il]) - n.klo[il]) * n.iw[il] : 0.0f;
    small = kf < n.kupu[0];
    tsm = ((kf - n.khi[0]) - n.klo[0]) * n.iw[m - 1];
}

// The same for a k_F clipped to kfclip (float64 value; only with a user bound).
__device__ __noinline__ void fz_member_clip(const FzRowArgs& a, int& il, float& til, bool& small, float& tsm) {
    const double kf = a.kfclip;
    const Member mb = membership(kf, a.kn, a.kup, a.m, true);
    il = mb.ilast;
    til = il >= 0 ? (float)(kf - a.kn[il]) / (float)(a.kn[il + 1] - a.kn[il]) : 0.0f;
    small = mb.small;
    tsm = (float)(kf - a.kn[0]) / (float)a.kn[0];
}

// Per-point interval of the interpolation: node fi gets 1 - tr and node fi + 1
// gets tr, both as max(0, 1 - |(j - fi) - tr|) for node j; fi = -2 when the
// point lies in no interval.  The small-k_F branch (node 0 only) is added
// separately at j = 0 (fz_small_weight).
__device__ __forceinline__ void fz_interval_state(float kf, const FzRowArgs& a, const FzNodeSm& n, float clipdn,
                                                  float& fi, float& tr) {
    int il;
    float til, tsm;
    bool small;
    if (kf > clipdn) fz_member_clip(a, il, til, small, tsm);
    else fz_member(kf, n, a.m, il, til, small, tsm);
    fi = il >= 0 ? (float)il : -2.0f;
    tr = il >= 0 ? til : 0.0f;
}

// Weight of node 0 from the small-k_F branch: pot1 takes it only at points in
// no interval (lwt.py:252-263); the hat planes add it to node 0 (lwt.py:266-296).
__device__ __forceinline__ float fz_small_weight(float kf, const FzRowArgs& a, const FzNodeSm& n, float clipdn,
                                                 bool only_outside) {
    int il;
    float til, tsm;
    bool small;
    if (kf > clipdn) fz_member_clip(a, il, til, small, tsm);
    else fz_member(kf, n, a.m, il, til, small, tsm);
    return (small && !(only_outside && il >= 0)) ? tsm : 0.0f;
}

__device__ __forceinline__ float fz_hat(float jf, float fi, float tr) {
    return fmaxf(0.0f, 1.0f - fabsf((jf - fi) - tr));
}

// Row l of a staged block (ROWS rows of H complex, then their ROWS Nyquist
// values) pre-processed for the half-length complex C2R:
// Z[k] = (X[k] + conj X[H-k]) + i w^k (X[k] - conj X[H-k]), w = exp(+2 pi i/n2),
// the imaginary parts of X[0] and X[H] dropped.
template <int H, int ROWS = kFzRowThreads / (H / kFzRowE)>
__device__ __forceinline__ void fz_c2r_pre(const float2* st, int l, int t, const float2* __restrict__ twr,
                                           float2 (&v)[kFzRowE]) {
    constexpr int E = kFzRowE, T = H / E;
    const float2* r = st + l * H;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k = t + T * e;
        float2 X = r[k];
        float2 Y = r[(H - k) & (H - 1)];
        if (e == 0 && k == 0) {
            Y = st[ROWS * H + l];
            X.y = 0.0f;
            Y.y = 0.0f;
        }
        const float2 A = make_float2(X.x + Y.x, X.y - Y.y);
        const float2 B = make_float2(X.x - Y.x, X.y + Y.y);
        const float2 wB = fz::cmulc(B, __ldg(twr + k));
        v[e] = make_float2(A.x - wB.y, A.y + wB.x);
    }
}

// shared memory of k_fz_c2r_rows (with_stages) and k_fz_r2c_rows
inline size_t fz_row_smem(int H, int m, bool with_stages) {
    const int T = H / kFzRowE, ROWS = kFzRowThreads / T;
    const size_t slots = (H + (H >> 4) + 1) + (H + 8 * (H >> 6) + 1);
    size_t b = 16 + (size_t)ROWS * slots * sizeof(float2) + (size_t)6 * m * sizeof(float);
    if (with_stages) b += 2 * (size_t)(ROWS * H + ROWS) * sizeof(float2);
    return b;
}

// Axis-2 C2R of the batch's planes plane0 .. plane0 + nb - 1 (node j0 + jj),
// row by row, interpolated into `pot` at every point of the row: pot1 from the
// P planes, pot3 from the M planes (SMALL: the small-k_F branch of node 0
// counts, which it does for pot1 only).  The block's rows of each plane (16 KB
// at n2 = 256) arrive by bulk copy two planes ahead of their use.
// HERM = 1 (P planes) or 2 (M planes): the cubic Hermite interpolation, whose
// P and M planes both feed pot1 and (kdd = 3) pot3 (fz_hermite_w); `pot` is
// then unused, and the M pass adds to what the P pass of the batch wrote.
template <int H, bool SMALL, int HERM = 0>
__global__ void __launch_bounds__(kFzRowThreads, 2) k_fz_c2r_rows(FzRowArgs a, int plane0, float* __restrict__ pot) {
    constexpr int E = kFzRowE, T = H / E, ROWS = kFzRowThreads / T, P = 2 * E;
    constexpr int STAGE = ROWS * H + ROWS;  // float2: the block's rows, then their Nyquist values
    using Lay = fz::RowLayout<H>;
    extern __shared__ float4 fz_rsm4[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(fz_rsm4);
    float2* stage = reinterpret_cast<float2*>(fz_rsm4 + 1);
    float2* buf0 = stage + 2 * STAGE;
    float2* buf1 = buf0 + ROWS * Lay::slots;
    float* fs = reinterpret_cast<float*>(buf1 + ROWS * Lay::slots1);
    const long long row0 = (long long)blockIdx.x * ROWS;
    auto issue = [&](int jj) {  // one thread: plane jj into stage jj & 1
        const int s = jj & 1;
        const float2* src = a.XY + (long long)(plane0 + jj) * a.d.plane;
        fz::mbar_expect_tx(&bar[s], STAGE * (unsigned)sizeof(float2));
        fz::bulk_load(stage + s * STAGE, src + row0 * H, ROWS * H * (unsigned)sizeof(float2), &bar[s]);
        fz::bulk_load(stage + s * STAGE + ROWS * H, src + a.d.nyq + row0, ROWS * (unsigned)sizeof(float2), &bar[s]);
    };
    __shared__ volatile int fail_flag;
    volatile int* fail = &fail_flag;
    int last_issued = -1;  // thread 0: the last plane whose copy it issued
    if (threadIdx.x == 0) {
        fail_flag = 0;
        fz::mbar_init(&bar[0], 1);
        fz::mbar_init(&bar[1], 1);
        fz::mbar_fence_init();
        issue(0);
        last_issued = 0;
        if (a.nb > 1) {
            issue(1);
            last_issued = 1;
        }
    }
    const FzNodeSm nodes = fz_stage_nodes(a, fs);
    __syncthreads();
    const int t = threadIdx.x % T, l = threadIdx.x / T;
    const long long row = row0 + l;
    const int n2 = 2 * H;
    float2* b0 = buf0 + l * Lay::slots;
    float2* b1 = buf1 + l * Lay::slots1;
    const typename Lay::Idx ix;
    const typename Lay::Idx1 ix1;
    const float clipdn = __double2float_rd(a.kfclip);
    const float2* kfrow = reinterpret_cast<const float2*>(a.kf + row * n2) + t;
    float fi[P], tr[P], acc[P];
    float acc3[HERM ? P : 1];
    const bool has3 = HERM && a.pot3 != nullptr;  // pot3 exists for kdd = 3 only
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const float2 kk = __ldg(kfrow + T * e);
        fz_interval_state(kk.x, a, nodes, clipdn, fi[2 * e], tr[2 * e]);
        fz_interval_state(kk.y, a, nodes, clipdn, fi[2 * e + 1], tr[2 * e + 1]);
        acc[2 * e] = acc[2 * e + 1] = 0.0f;
        if constexpr (HERM != 0) acc3[2 * e] = acc3[2 * e + 1] = 0.0f;
    }
    // register twiddles, except for the Hermite passes (their second accumulator takes the registers)
    float2 twr[HERM ? 1 : fz::tw_count<H, E>()];
    if constexpr (HERM == 0) fz::tw_load<H, E>(twr, t, a.tw.th);
    for (int jj = 0; jj < a.nb; ++jj) {
        const int j = a.j0 + jj;
        const int s = jj & 1;
        // a copy that did not complete in time sets the error word and the block's
        // flag; later waits are skipped, no more copies are issued, and the copies
        // in flight are drained after the loop (the results are then garbage and
        // the host raises the error).  Every thread runs the same barriers either way.
        if (!*fail && !fz::mbar_wait(&bar[s], (jj >> 1) & 1)) {
            *fail = 1;
            atomicOr(a.err, 1u);
        }
        float2 v[E];
        fz_c2r_pre<H>(stage + s * STAGE, l, t, a.tw.tr, v);
        if constexpr (HERM == 0) fz::line_fft_ppr<H, E, +1>(v, b0, b1, ix, ix1, t, twr);
        else fz::line_fft_pp<H, E, +1>(v, b0, b1, ix, t, a.tw.th);
        // every thread has passed the transform's first barrier, so stage s is read
        if (threadIdx.x == 0 && jj + 2 < a.nb && !*fail) {
            fz::fence_proxy_async();
            issue(jj + 2);
            last_issued = jj + 2;
        }
        const float jf = (float)j;
        if constexpr (HERM == 0) {
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const float pv = (q & 1) ? v[q >> 1].y : v[q >> 1].x;
                acc[q] = fmaf(fz_hat(jf, fi[q], tr[q]), pv, acc[q]);
            }
        } else {
            const float D0 = nodes.dk[j], D1 = j > 0 ? nodes.dk[j - 1] : 0.0f;
            const float iD0 = D0 > 0.0f ? 1.0f / D0 : 0.0f, iD1 = D1 > 0.0f ? 1.0f / D1 : 0.0f;
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const float pv = (q & 1) ? v[q >> 1].y : v[q >> 1].x;
                const float dd = jf - fi[q];
                float w1, w3;
                fz_hermite_w<HERM == 2>(tr[q], dd == 0.0f, dd == 1.0f, D0, D1, iD0, iD1, w1, w3);
                acc[q] = fmaf(w1, pv, acc[q]);
                if (has3) acc3[q] = fmaf(w3, pv, acc3[q]);
            }
        }
        if (SMALL && j == 0) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const float2 kk = __ldg(kfrow + T * e);
                acc[2 * e] = fmaf(fz_small_weight(kk.x, a, nodes, clipdn, true), v[e].x, acc[2 * e]);
                acc[2 * e + 1] = fmaf(fz_small_weight(kk.y, a, nodes, clipdn, true), v[e].y, acc[2 * e + 1]);
            }
        }
    }
    if (threadIdx.x == 0 && *fail) {
        // let the copies still in flight land before the block exits (bounded)
        for (int q = (last_issued > 0 ? last_issued - 1 : 0); q <= last_issued; ++q)
            fz::mbar_wait(&bar[q & 1], (q >> 1) & 1);
    }
    // the P pass of a first batch writes; every other pass adds
    const bool add = !a.first || HERM == 2;
    float* const pot1 = HERM ? a.pot1 : pot;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        float2* p = reinterpret_cast<float2*>(pot1 + row * n2) + t + T * e;
        float2 o = make_float2(acc[2 * e], acc[2 * e + 1]);
        if (add) {
            const float2 old = *p;
            o = make_float2(old.x + o.x, old.y + o.y);
        }
        *p = o;
        if constexpr (HERM != 0) {
            if (has3) {
                float2* p3 = reinterpret_cast<float2*>(a.pot3 + row * n2) + t + T * e;
                float2 o3 = make_float2(acc3[2 * e], acc3[2 * e + 1]);
                if (add) {
                    const float2 old = *p3;
                    o3 = make_float2(old.x + o3.x, old.y + o3.y);
                }
                *p3 = o3;
            }
        }
    }
}

// rho^alpha W_j of every node of the batch, R2C along axis 2, row by row.
// The post-processing pairs (k, H-k) are exchanged between the row's threads
// with shuffles: element H-k of thread t's slot e sits in thread (T - t) % T,
// slot E-1-e (t > 0) or in thread 0, slot (E-e) % E (t = 0).
// HERM: the cubic Hermite interpolation's two hat planes per node, rho^alpha
// times h00 | h01 into plane jj and rho^alpha times D0 h10 | D1 h11 into plane
// nb + jj (lwt.py:285-296; fz_hermite_w's w1 of the P and M planes).
template <int H, bool HERM = false>
__global__ void __launch_bounds__(kFzRowThreads, 2) k_fz_r2c_rows(FzRowArgs a) {
    constexpr int E = kFzRowE, T = H / E, ROWS = kFzRowThreads / T, P = 2 * E;
    static_assert(T <= 32, "a row must fit in one warp");
    using Lay = fz::RowLayout<H>;
    extern __shared__ float4 fz_rsm4[];
    float2* buf0 = reinterpret_cast<float2*>(fz_rsm4 + 1);
    float2* buf1 = buf0 + ROWS * Lay::slots;
    float* fs = reinterpret_cast<float*>(buf1 + ROWS * Lay::slots1);
    const FzNodeSm nodes = fz_stage_nodes(a, fs);
    __syncthreads();
    const int t = threadIdx.x % T, l = threadIdx.x / T;
    const long long row = (long long)blockIdx.x * ROWS + l;
    const int n2 = 2 * H;
    float2* b0 = buf0 + l * Lay::slots;
    float2* b1 = buf1 + l * Lay::slots1;
    const typename Lay::Idx ix;
    const typename Lay::Idx1 ix1;
    const float clipdn = __double2float_rd(a.kfclip);
    const int lane = threadIdx.x & 31;
    const int partner = (lane & ~(T - 1)) | ((T - t) & (T - 1));
    const float2* kfrow = reinterpret_cast<const float2*>(a.kf + row * n2) + t;
    const float2* rarow = reinterpret_cast<const float2*>(a.rA + row * n2) + t;
    // rho^alpha of the thread's points in registers (with the Hermite planes: read again per node)
    float fi[P], tr[P], ra_r[HERM ? 1 : P];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const float2 kk = __ldg(kfrow + T * e);
        fz_interval_state(kk.x, a, nodes, clipdn, fi[2 * e], tr[2 * e]);
        fz_interval_state(kk.y, a, nodes, clipdn, fi[2 * e + 1], tr[2 * e + 1]);
        if constexpr (!HERM) {
            const float2 rr = __ldg(rarow + T * e);
            ra_r[2 * e] = rr.x;
            ra_r[2 * e + 1] = rr.y;
        }
    }
    auto ra = [&](int q) {
        if constexpr (HERM) {
            const float2 rr = __ldg(rarow + T * (q >> 1));
            return (q & 1) ? rr.y : rr.x;
        } else {
            return ra_r[q];
        }
    };
    // register twiddles, except with the Hermite planes (the two transforms per node take the registers)
    float2 twr[HERM ? 1 : fz::tw_count<H, E>()];
    if constexpr (!HERM) fz::tw_load<H, E>(twr, t, a.tw.th);
    // the row transform of v, post-processed and stored into plane pl
    auto emit = [&](float2 (&v)[E], int pl) {
        if constexpr (!HERM) fz::line_fft_ppr<H, E, -1>(v, b0, b1, ix, ix1, t, twr);
        else fz::line_fft_pp<H, E, -1>(v, b0, b1, ix, t, a.tw.th);
        float2* dst = a.XY + (long long)pl * a.d.plane;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int k = t + T * e;
            const float2 Zk = v[e];
            float2 Zc;
            Zc.x = __shfl_sync(0xffffffffu, v[E - 1 - e].x, partner);
            Zc.y = __shfl_sync(0xffffffffu, v[E - 1 - e].y, partner);
            if (t == 0) Zc = v[(E - e) % E];
            // X = (Zk + conj Zc)/2 - i w^-k (Zk - conj Zc)/2, w^-k = exp(-2 pi i k/n2)
            const float2 A = make_float2(0.5f * (Zk.x + Zc.x), 0.5f * (Zk.y - Zc.y));
            const float2 B = make_float2(0.5f * (Zk.x - Zc.x), 0.5f * (Zk.y + Zc.y));
            const float2 wB = fz::cmul(B, __ldg(a.tw.tr + k));
            __stcs(dst + row * H + k, make_float2(A.x + wB.y, A.y - wB.x));
        }
        if (t == 0) __stcs(dst + a.d.nyq + row, make_float2(v[0].x - v[0].y, 0.0f));
    };
    for (int jj = 0; jj < a.nb; ++jj) {
        const int j = a.j0 + jj;
        const float jf = (float)j;
        float2 v[E];
        float D0 = 0.0f, D1 = 0.0f;
        if constexpr (HERM) {
            D0 = nodes.dk[j];
            D1 = j > 0 ? nodes.dk[j - 1] : 0.0f;
        }
        // hat weight of node j at point q: linear, or the P planes' w1 of the Hermite interpolation
        auto wP = [&](int q) {
            if constexpr (HERM) {
                const float dd = jf - fi[q];
                float w1, w3;
                fz_hermite_w<false>(tr[q], dd == 0.0f, dd == 1.0f, D0, D1, 0.0f, 0.0f, w1, w3);
                return w1;
            } else {
                return fz_hat(jf, fi[q], tr[q]);
            }
        };
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = make_float2(ra(2 * e) * wP(2 * e), ra(2 * e + 1) * wP(2 * e + 1));
        if (j == 0) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const float2 kk = __ldg(kfrow + T * e);
                v[e].x = fmaf(ra(2 * e), fz_small_weight(kk.x, a, nodes, clipdn, false), v[e].x);
                v[e].y = fmaf(ra(2 * e + 1), fz_small_weight(kk.y, a, nodes, clipdn, false), v[e].y);
            }
        }
        emit(v, jj);
        if constexpr (HERM) {
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const float dd = jf - fi[q];
                float w1, w3;
                fz_hermite_w<true>(tr[q], dd == 0.0f, dd == 1.0f, D0, D1, 0.0f, 0.0f, w1, w3);
                if (q & 1) v[q >> 1].y = ra(q) * w1;
                else v[q >> 1].x = ra(q) * w1;
            }
            emit(v, a.nb + jj);
        }
    }
}

// Axis-0 forward transform of the batch's planes, K_j(G)/N applied and summed
// into pot2(G) (lwt.py:266-296; the sum starts from the previous batches').
// K_j(0) = 0: the G = 0 element keeps its starting value.  HERM: plane nb + jj
// (the Hermite interpolation's second hat plane) adds K'_j(G)/k_j/N times its
// transform, the M planes' kernel.
template <int N0, bool HERM = false>
__global__ void __launch_bounds__(kFzLines * (N0 / kFzColE), 2)
    k_fz_pot2(const float2* __restrict__ XY, float2* __restrict__ pot2G, FzTab tb, const double* __restrict__ knode,
              const double* __restrict__ invk, int j0, int nb, int first, Geo geo, FzDims d,
              const float2* __restrict__ tw, float invN) {
    constexpr int E = kFzColE, T = N0 / E, L = kFzLines;
    extern __shared__ float2 fz_sm[];
    float2* sm = fz_sm;
    float* sq = reinterpret_cast<float*>(fz_sm + fz::col_slots(N0));
    float* siq = sq + N0 * L;
    float* sik = siq + N0 * L;
    float* sk2 = sik + nb;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        const double k = knode[j0 + q];
        sik[q] = (float)invk[j0 + q];
        sk2[q] = (float)(k * k);
    }
    const int l = threadIdx.x % L, t = threadIdx.x / L;
    int k1, k2;
    long long pbase, pstride, gbase, gstride;
    fz_axis0_tile(d, blockIdx.x, l, k1, k2, pbase, pstride, gbase, gstride);
    float2 acc[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k0 = t + T * e;
        const int s = k0 * L + l;
        const float q2 = gsq_f(geo, k0, k1, k2);
        sq[s] = sqrtf(q2);
        siq[s] = q2 > 0.0f ? 1.0f / q2 : 0.0f;
        acc[e] = first ? make_float2(0.0f, 0.0f) : pot2G[gbase + k0 * gstride];
    }
    const bool g0 = (t == 0 && k1 == 0 && k2 == 0);
    const float2 acc00 = acc[0];
    // register twiddles, except with the Hermite planes (two transforms per node)
    float2 twr[HERM ? 1 : fz::tw_count<N0, E>()];
    if constexpr (!HERM) fz::tw_load<N0, E>(twr, t, tw);
    float qmin = INFINITY;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k0 = t + T * e;
        qmin = fminf(qmin, sqrtf(gsq_f(geo, k0, k1, k2)));
    }
    qmin = fz_warp_min(qmin);
    // plane pl transformed along axis 0, times the node kernel of node jj (DERIV: K'_j/k_j), into acc
    auto accumulate = [&](int pl, int jj, auto deriv) {
        constexpr bool DERIV = decltype(deriv)::value;
        const float2* inp = XY + (long long)pl * d.plane + pbase;
        float2 v[E];
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = __ldcs(inp + (t + T * e) * pstride);
        __syncthreads();  // the exchange buffer is free; the node and |G| tables are staged
        if constexpr (!HERM) fz::line_fft_r<N0, E, -1>(v, sm + l, fz::ColIdx(), t, twr);
        else fz::line_fft<N0, E, -1>(v, sm + l, fz::ColIdx(), t, tw);
        const float ik = sik[jj], kj2 = sk2[jj];
        if constexpr (!HERM) {
            float f[E];
            auto factors = [&](auto near) {
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const int s = (t + T * e) * L + l;
                    const float kv = fz_node_kernel<DERIV, decltype(near)::value>(tb, sq[s], ik, siq[s], kj2);
                    f[e] = (DERIV ? kv * ik : kv) * invN;
                }
            };
            // warp-uniform: does any point of this warp need the spline for node j?
            if (qmin * ik < tb.eta_series) factors(std::true_type());
            else factors(std::false_type());
#pragma unroll
            for (int e = 0; e < E; ++e) {
                acc[e].x = fmaf(f[e], v[e].x, acc[e].x);
                acc[e].y = fmaf(f[e], v[e].y, acc[e].y);
            }
        } else {
            // each factor goes into the sum at once (fewer live registers beside two transforms per node)
            auto factors = [&](auto near) {
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const int s = (t + T * e) * L + l;
                    const float kv = fz_node_kernel<DERIV, decltype(near)::value>(tb, sq[s], ik, siq[s], kj2);
                    const float f = (DERIV ? kv * ik : kv) * invN;
                    acc[e].x = fmaf(f, v[e].x, acc[e].x);
                    acc[e].y = fmaf(f, v[e].y, acc[e].y);
                }
            };
            if (qmin * ik < tb.eta_series) factors(std::true_type());
            else factors(std::false_type());
        }
    };
    if constexpr (!HERM) {
        for (int jj = 0; jj < nb; ++jj) accumulate(jj, jj, std::false_type());
    } else {
        // one loop body over the 2 nb planes (node jj's planes jj and nb + jj in turn)
        for (int pp = 0; pp < 2 * nb; ++pp) {
            const int jj = pp >> 1;
            if (pp & 1) accumulate(nb + jj, jj, std::true_type());
            else accumulate(jj, jj, std::false_type());
        }
    }
    if (g0) acc[0] = acc00;
#pragma unroll
    for (int e = 0; e < E; ++e) pot2G[gbase + (t + T * e) * gstride] = acc[e];
}

}  // namespace
