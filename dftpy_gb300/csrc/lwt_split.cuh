// The fused float32 k_F-node pipeline with axis 1 split between the two passes
// of each chain, for grids with n1 = n2 = 256 (n0 any tile-FFT length), so
// that neither chain has an axis-1 plane pass and every node plane crosses HBM
// twice (written once, read once) instead of four times.
//
// The 256-point transform along axis 1 runs as radix 8 x 32: with
// k1 = a + 32 b and r1 = d + 8 c (a, c < 32; b, d < 8) and w_n = exp(2 pi i/n),
//   inverse  y[d + 8 c]  = sum_a w_32^{ac}  (w_256^{ad}  sum_b x[a + 32 b] w_8^{bd})
//   forward  X[a + 32 b] = sum_d w_8^{-bd} (w_256^{-ad} sum_c x[d + 8 c] w_32^{-ac})
// Between the passes a plane holds axis-1 element (d, a) at row 32 d + a of the
// usual [n0][256][H] block (Nyquist [n0][256]), so the 32 values a of one
// (i0, d) are 32 consecutive rows: one contiguous 32 KB block.
//   C2R: k_fz_n8      node kernel on load, axis 0, the radix-8 stage over b
//                     with the w_256 twiddles; full 32-byte sectors stored
//        k_fz_c2r_s8  per (i0, d): the 32-point stage over a, then the axis-2
//                     C2R of rows r1 = d + 8 c and the interpolation
//   R2C: k_fz_r2c_s8  per (i0, d): hat weights, axis-2 R2C of rows d + 8 c,
//                     the 32-point stage over c with the w_256 twiddles
//        k_fz_pot2_s8 the radix-8 stage over d, axis 0, node kernel, pot2(G)
// The arithmetic is that of k_fz_nodes / k_fz_axis1 / k_fz_c2r_rows (and of
// k_fz_r2c_rows / k_fz_axis1 / k_fz_pot2) with the axis-1 transform factored
// differently, so results agree with those kernels to float32 round-off.
#pragma once
#include "lwt_fused.cuh"

namespace {

constexpr int kS8L = 32;     // lines of a split column tile: line l = 4 b + c
constexpr int kS8P = 36;     // pitch (float2) of the radix-8 exchange rows: 32 lines + 4
constexpr int kS8Rows = 32;  // rows of a split row block (the 32 values of a or c)
constexpr int kS8RowThreads = kS8Rows * (128 / kFzRowE);

// Column tile of the split passes: main tiles (a0, q) take lines l = 4 b + c at
// k1 = a0 + 32 b, k2 = 4 q + c (q fastest: neighbouring tiles fill neighbouring
// sectors); Nyquist tiles take k1 = a0 + c + 32 b with a0 = 4 q', k2 = H.
__device__ __forceinline__ void fz8_tile(const FzDims& d, int tile, int& a0, int& q, bool& nyq) {
    const int per = d.H / 4, tiles_main = 32 * per;
    nyq = tile >= tiles_main;
    a0 = nyq ? 4 * (tile - tiles_main) : tile / per;
    q = nyq ? 0 : tile % per;
}
inline int fz8_tiles(int H) { return 32 * (H / 4) + 8; }

// axis-0 exchange of a split column tile: element n of line l at n * 32 + l
struct S8ColIdx {
    __device__ __forceinline__ int operator()(int n) const { return n * kS8L; }
};
// 32-point exchange of a split row block: element n of column col at n * 128 + col
struct S8RowIdx {
    __device__ __forceinline__ int operator()(int n) const { return n * 128; }
};

// 16-byte asynchronous copy global -> shared (both addresses 16-byte aligned),
// completed by cp_async_wait_all in the copying thread
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(fz::smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// k_fz_n8: radix-8 exchange, staged FFT(rho^beta)/N, |G|, 1/|G|^2, node tables
inline size_t fz8_nodes_smem(int n0, int nb) {
    const size_t pts = (size_t)n0 * kS8L;
    return (size_t)n0 * kS8P * sizeof(float2) + pts * (sizeof(float2) + 2 * sizeof(float)) +
           2 * (size_t)nb * sizeof(float);
}
// k_fz_pot2_s8: radix-8 exchange, axis-0 exchange, |G|, 1/|G|^2, node tables
inline size_t fz8_pot2_smem(int n0, int nb) { return fz8_nodes_smem(n0, nb); }
// k_fz_c2r_s8 (two stages for the bulk copies) and k_fz_r2c_s8 (one)
inline size_t fz8_row_smem(int m, int stages) {
    using Lay = fz::RowLayout<128>;
    return 16 + (size_t)stages * (kS8Rows * 128 + kS8Rows) * sizeof(float2) +
           (size_t)kS8Rows * (Lay::slots + Lay::slots1) * sizeof(float2) + (size_t)6 * m * sizeof(float);
}

// The 32-point transform (sign S) along the row index of a staged row block
// st (kS8Rows rows of 128 complex): thread tid takes column tid & 127 and
// returns its elements cq + 4 e in u[e] (cq = tid >> 7), exchanging through
// xb.  Entry: xb free.  On return every thread has read its inputs from st.
template <int S>
__device__ __forceinline__ void fz8_col32(const float2* st, float2* xb, const float2* __restrict__ tq,
                                          float2 (&u)[8]) {
    const int col = threadIdx.x & 127, cq = threadIdx.x >> 7;
#pragma unroll
    for (int e = 0; e < 8; ++e) u[e] = st[(cq + 4 * e) * 128 + col];
    fz::line_fft<32, 8, S>(u, xb + col, S8RowIdx(), cq, tq);
}
// The same transform of the block's 32 Nyquist values nq by one warp: lane n
// loads element n, five radix-2 decimation-in-frequency stages exchange
// through shuffles (stage span h: lanes with bit h clear keep x + x', lanes
// with it set keep (x' - x) w^((n mod h) 16/h)), which leaves output
// bitrev(n) in lane n; a last shuffle returns output c to lane c.
template <int S>
__device__ __forceinline__ float2 fz8_nyq32(const float2* nq, const float2* __restrict__ tq) {
    const int n = threadIdx.x & 31;
    float2 w[4];  // stages h = 16, 8, 4, 2 (h = 1 has no twiddle)
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int h = 16 >> s;
        w[s] = __ldg(tq + (n & (h - 1)) * (16 / h));
    }
    float2 x = nq[n];
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        const int h = 16 >> s;
        float2 y;
        y.x = __shfl_xor_sync(0xffffffffu, x.x, h);
        y.y = __shfl_xor_sync(0xffffffffu, x.y, h);
        if (n & h) {
            const float2 dlt = fz::csub(y, x);
            x = s < 4 ? (S < 0 ? fz::cmul(dlt, w[s]) : fz::cmulc(dlt, w[s])) : dlt;
        } else {
            x = fz::cadd(x, y);
        }
    }
    const int src = __brev(n) >> 27;  // the lane holding output n
    float2 o;
    o.x = __shfl_sync(0xffffffffu, x.x, src);
    o.y = __shfl_sync(0xffffffffu, x.y, src);
    return o;
}

// The node kernel on load (as k_fz_nodes), the axis-0 inverse transform, then
// the radix-8 stage over b into plane plane0 + jj of the split layout.
template <int N0, bool DERIV>
__global__ void __launch_bounds__(kS8L*(N0 / kFzColE), 1)
    k_fz_n8(const float2* __restrict__ rbG, float2* __restrict__ XY, FzTab tb, const double* __restrict__ knode,
            const double* __restrict__ invk, int j0, int nb, int plane0, Geo geo, FzDims d,
            const float2* __restrict__ tw0, const float2* __restrict__ tw1, float invN) {
    constexpr int E = kFzColE, T = N0 / E, L = kS8L, NT = L * T;
    static_assert(NT == 2 * N0, "two (r0, c) pairs per thread in the radix-8 stage");
    extern __shared__ float2 fz_sm[];
    float2* X = fz_sm;
    float2* sz = X + N0 * kS8P;
    float* sq = reinterpret_cast<float*>(sz + N0 * L);
    float* siq = sq + N0 * L;
    float* sik = siq + N0 * L;
    float* sk2 = sik + nb;
    for (int i = threadIdx.x; i < nb; i += NT) {
        const double k = knode[j0 + i];
        sik[i] = (float)invk[j0 + i];
        sk2[i] = (float)(k * k);
    }
    int a0, q;
    bool nyq;
    fz8_tile(d, blockIdx.x, a0, q, nyq);
    const int l = threadIdx.x % L, t = threadIdx.x / L;
    {
        const int b = l >> 2, c = l & 3;
        const int k1 = (nyq ? a0 + c : a0) + 32 * b, k2 = nyq ? d.H : 4 * q + c;
        const long long gbase = (long long)k1 * (d.H + 1) + k2, gstride = (long long)d.n1 * (d.H + 1);
#pragma unroll 4
        for (int e = 0; e < E; ++e) {
            const int k0 = t + T * e;
            const int s = k0 * L + l;
            float2 z = __ldg(rbG + gbase + k0 * gstride);
            z = make_float2(z.x * invN, z.y * invN);
            const float q2 = gsq_f(geo, k0, k1, k2);
            if (k0 == 0 && k1 == 0 && k2 == 0) z = make_float2(0.0f, 0.0f);
            sz[s] = z;
            sq[s] = sqrtf(q2);
            siq[s] = q2 > 0.0f ? 1.0f / q2 : 0.0f;
        }
    }
    float2 twr[fz::tw_count<N0, E>()];
    fz::tw_load<N0, E>(twr, t, tw0);
    // radix-8 stage: thread tid takes the pairs (r0, c) = (p >> 2, p & 3) of
    // p = tid and tid + NT; both have c = tid & 3, and a = a0 (+ c on Nyquist tiles)
    const int pc = threadIdx.x & 3;
    const int pa = nyq ? a0 + pc : a0;
    float2 w8[7];
#pragma unroll
    for (int dd = 1; dd < 8; ++dd) w8[dd - 1] = __ldg(tw1 + ((pa * dd) & (d.n1 - 1)));
    const long long ostep = nyq ? 32 : 32LL * d.H;                            // per d
    const long long obase = nyq ? d.nyq + pa : (long long)pa * d.H + 4 * q + pc;
    const long long ostride = nyq ? d.n1 : (long long)d.n1 * d.H;             // per r0
    __syncthreads();
    float qmin = INFINITY;
#pragma unroll
    for (int e = 0; e < E; ++e) qmin = fminf(qmin, sq[(t + T * e) * L + l]);
    qmin = fz_warp_min(qmin);
    for (int jj = 0; jj < nb; ++jj) {
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
        __syncthreads();  // X is free: every thread has read the previous node's pairs
        fz::line_fft_r<N0, E, +1>(v, X + l, S8ColIdx(), t, twr);
        __syncthreads();  // the transform's last reads of X are done
#pragma unroll
        for (int e = 0; e < E; ++e) X[(t + T * e) * kS8P + l] = v[e];
        __syncthreads();
        float2* outp = XY + (long long)(plane0 + jj) * d.plane + obase;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r0 = (threadIdx.x + NT * h) >> 2;
            float2 u[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) u[b] = X[r0 * kS8P + 4 * b + pc];
            fz::dft8<+1>(u);
#pragma unroll
            for (int dd = 1; dd < 8; ++dd) u[dd] = fz::cmulc(u[dd], w8[dd - 1]);
#pragma unroll
            for (int dd = 0; dd < 8; ++dd) __stcs(outp + r0 * ostride + dd * ostep, u[dd]);
        }
    }
}

// C2R consumer of the split layout: block (i0, d) takes the 32 rows
// (i0, 32 d + a) of each plane by bulk copy two planes ahead, runs the
// 32-point stage over a in place, and then, as k_fz_c2r_rows, the axis-2 C2R
// of rows r1 = d + 8 c and the interpolation into pot (SMALL as there).
template <bool SMALL>
__global__ void __launch_bounds__(kS8RowThreads, 1) k_fz_c2r_s8(FzRowArgs a, int plane0, float* __restrict__ pot) {
    constexpr int H = 128, E = kFzRowE, T = H / E, ROWS = kS8Rows, P = 2 * E;
    constexpr int STAGE = ROWS * H + ROWS;
    static_assert(ROWS * T == kS8RowThreads && kS8RowThreads == 4 * H, "one thread per (row, sixteenth of a row)");
    using Lay = fz::RowLayout<H>;
    extern __shared__ float4 fz_rsm4[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(fz_rsm4);
    float2* stage = reinterpret_cast<float2*>(fz_rsm4 + 1);
    float2* buf0 = stage + 2 * STAGE;
    float2* buf1 = buf0 + ROWS * Lay::slots;
    float* fs = reinterpret_cast<float*>(buf1 + ROWS * Lay::slots1);
    const int i0 = blockIdx.x >> 3, dd = blockIdx.x & 7;
    const long long prow0 = (long long)i0 * a.d.n1 + 32 * dd;  // plane row of a = 0
    auto issue = [&](int jj) {  // one thread: plane jj into stage jj & 1
        const int s = jj & 1;
        const float2* src = a.XY + (long long)(plane0 + jj) * a.d.plane;
        fz::mbar_expect_tx(&bar[s], STAGE * (unsigned)sizeof(float2));
        fz::bulk_load(stage + s * STAGE, src + prow0 * H, ROWS * H * (unsigned)sizeof(float2), &bar[s]);
        fz::bulk_load(stage + s * STAGE + ROWS * H, src + a.d.nyq + prow0, ROWS * (unsigned)sizeof(float2), &bar[s]);
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
    const long long row = (long long)i0 * a.d.n1 + dd + 8 * l;  // r1 = d + 8 c with c = l
    const int n2 = 2 * H;
    float2* b0 = buf0 + l * Lay::slots;
    float2* b1 = buf1 + l * Lay::slots1;
    const typename Lay::Idx ix;
    const typename Lay::Idx1 ix1;
    const float clipdn = __double2float_rd(a.kfclip);
    const float2* kfrow = reinterpret_cast<const float2*>(a.kf + row * n2) + t;
    float fi[P], tr[P], acc[P];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const float2 kk = __ldg(kfrow + T * e);
        fz_interval_state(kk.x, a, nodes, clipdn, fi[2 * e], tr[2 * e]);
        fz_interval_state(kk.y, a, nodes, clipdn, fi[2 * e + 1], tr[2 * e + 1]);
        acc[2 * e] = acc[2 * e + 1] = 0.0f;
    }
    float2 twr[fz::tw_count<H, E>()];
    fz::tw_load<H, E>(twr, t, a.tw.th);
    const int col = threadIdx.x & (H - 1), cq = threadIdx.x >> 7;
    for (int jj = 0; jj < a.nb; ++jj) {
        const int j = a.j0 + jj;
        const int s = jj & 1;
        // a copy that did not complete in time: as k_fz_c2r_rows
        if (!*fail && !fz::mbar_wait(&bar[s], (jj >> 1) & 1)) {
            *fail = 1;
            atomicOr(a.err, 1u);
        }
        float2* st = stage + s * STAGE;
        {
            // the 32-point stage over a, in place: column col's outputs c = cq + 4 e
            float2 u[8];
            fz8_col32<+1>(st, buf0, a.tw.tq, u);
            float2 un = make_float2(0.0f, 0.0f);
            if (threadIdx.x < 32) un = fz8_nyq32<+1>(st + ROWS * H, a.tw.tq);
#pragma unroll
            for (int e = 0; e < 8; ++e) st[(cq + 4 * e) * H + col] = u[e];
            if (threadIdx.x < 32) {
                __syncwarp();
                st[ROWS * H + threadIdx.x] = un;
            }
        }
        __syncthreads();  // rows r1 = d + 8 c are in st; every thread is done with buf0
        float2 v[E];
        fz_c2r_pre<H, ROWS>(st, l, t, a.tw.tr, v);
        fz::fence_proxy_async();  // this thread's accesses to st come before the next copy into it
        fz::line_fft_ppr<H, E, +1>(v, b0, b1, ix, ix1, t, twr);
        // every thread has passed the transform's first barrier, so stage s is read
        if (threadIdx.x == 0 && jj + 2 < a.nb && !*fail) {
            issue(jj + 2);
            last_issued = jj + 2;
        }
        const float jf = (float)j;
#pragma unroll
        for (int qq = 0; qq < P; ++qq) {
            const float pv = (qq & 1) ? v[qq >> 1].y : v[qq >> 1].x;
            acc[qq] = fmaf(fz_hat(jf, fi[qq], tr[qq]), pv, acc[qq]);
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
        for (int qq = (last_issued > 0 ? last_issued - 1 : 0); qq <= last_issued; ++qq)
            fz::mbar_wait(&bar[qq & 1], (qq >> 1) & 1);
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
        float2* p = reinterpret_cast<float2*>(pot + row * n2) + t + T * e;
        float2 o = make_float2(acc[2 * e], acc[2 * e + 1]);
        if (!a.first) {
            const float2 old = *p;
            o = make_float2(old.x + o.x, old.y + o.y);
        }
        *p = o;
    }
}

// R2C of the split layout: block (i0, d) forms rho^alpha W_j on rows
// r1 = d + 8 c (c < 32) for every node of the batch, transforms them along
// axis 2 (as k_fz_r2c_rows), then along c (the 32-point stage, w_256^{-a d}
// applied), and stores rows (i0, 32 d + a) of plane jj.
__global__ void __launch_bounds__(kS8RowThreads, 1) k_fz_r2c_s8(FzRowArgs a) {
    constexpr int H = 128, E = kFzRowE, T = H / E, ROWS = kS8Rows, P = 2 * E;
    static_assert(T <= 32, "a row must fit in one warp");
    using Lay = fz::RowLayout<H>;
    extern __shared__ float4 fz_rsm4[];
    float2* S = reinterpret_cast<float2*>(fz_rsm4 + 1);  // [ROWS][H], then the ROWS Nyquist values
    float2* buf0 = S + ROWS * H + ROWS;
    float2* buf1 = buf0 + ROWS * Lay::slots;
    float* fs = reinterpret_cast<float*>(buf1 + ROWS * Lay::slots1);
    const FzNodeSm nodes = fz_stage_nodes(a, fs);
    __syncthreads();
    const int i0 = blockIdx.x >> 3, dd = blockIdx.x & 7;
    const int t = threadIdx.x % T, l = threadIdx.x / T;
    const long long row = (long long)i0 * a.d.n1 + dd + 8 * l;  // r1 = d + 8 c with c = l
    const long long prow0 = (long long)i0 * a.d.n1 + 32 * dd;   // plane row of a = 0
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
    float fi[P], tr[P], ra[P];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const float2 kk = __ldg(kfrow + T * e);
        const float2 rr = __ldg(rarow + T * e);
        fz_interval_state(kk.x, a, nodes, clipdn, fi[2 * e], tr[2 * e]);
        fz_interval_state(kk.y, a, nodes, clipdn, fi[2 * e + 1], tr[2 * e + 1]);
        ra[2 * e] = rr.x;
        ra[2 * e + 1] = rr.y;
    }
    float2 twr[fz::tw_count<H, E>()];
    fz::tw_load<H, E>(twr, t, a.tw.th);
    // the 32-point stage: thread tid's outputs a = cq + 4 e of column col, times w_256^{-a d}
    const int col = threadIdx.x & (H - 1), cq = threadIdx.x >> 7;
    __shared__ float2 w32[32];  // w_256^{-a d}, a < 32
    if (threadIdx.x < 32) w32[threadIdx.x] = __ldg(a.tw.t1 + ((threadIdx.x * dd) & (a.d.n1 - 1)));
    for (int jj = 0; jj < a.nb; ++jj) {
        const int j = a.j0 + jj;
        const float jf = (float)j;
        float2 v[E];
#pragma unroll
        for (int e = 0; e < E; ++e)
            v[e] = make_float2(ra[2 * e] * fz_hat(jf, fi[2 * e], tr[2 * e]),
                               ra[2 * e + 1] * fz_hat(jf, fi[2 * e + 1], tr[2 * e + 1]));
        if (j == 0) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const float2 kk = __ldg(kfrow + T * e);
                v[e].x = fmaf(ra[2 * e], fz_small_weight(kk.x, a, nodes, clipdn, false), v[e].x);
                v[e].y = fmaf(ra[2 * e + 1], fz_small_weight(kk.y, a, nodes, clipdn, false), v[e].y);
            }
        }
        __syncthreads();  // buf0 and S are free: the previous node's 32-point stage has read them
        fz::line_fft_ppr<H, E, -1>(v, b0, b1, ix, ix1, t, twr);
        // R2C post-processing as k_fz_r2c_rows, into S
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int k = t + T * e;
            const float2 Zk = v[e];
            float2 Zc;
            Zc.x = __shfl_sync(0xffffffffu, v[E - 1 - e].x, partner);
            Zc.y = __shfl_sync(0xffffffffu, v[E - 1 - e].y, partner);
            if (t == 0) Zc = v[(E - e) % E];
            const float2 A = make_float2(0.5f * (Zk.x + Zc.x), 0.5f * (Zk.y - Zc.y));
            const float2 B = make_float2(0.5f * (Zk.x - Zc.x), 0.5f * (Zk.y + Zc.y));
            const float2 wB = fz::cmul(B, __ldg(a.tw.tr + k));
            S[l * H + k] = make_float2(A.x + wB.y, A.y - wB.x);
        }
        if (t == 0) S[ROWS * H + l] = make_float2(v[0].x - v[0].y, 0.0f);
        __syncthreads();  // the block's row spectra are in S
        float2 u[8];
        fz8_col32<-1>(S, buf0, a.tw.tq, u);
        float2* dst = a.XY + (long long)jj * a.d.plane;
#pragma unroll
        for (int e = 0; e < 8; ++e) __stcs(dst + (prow0 + cq + 4 * e) * H + col, fz::cmul(u[e], w32[cq + 4 * e]));
        if (threadIdx.x < 32) {
            const float2 un = fz8_nyq32<-1>(S + ROWS * H, a.tw.tq);
            __stcs(dst + a.d.nyq + prow0 + lane, fz::cmul(un, w32[lane]));
        }
    }
}

// The radix-8 stage over d of the split layout, the axis-0 forward transform,
// K_j(G)/N applied and summed into pot2(G) (as k_fz_pot2; the sum starts from
// the previous batches', and the G = 0 element keeps its starting value).
// Each node's tile (the 32-byte pieces of rows 32 d + a0 at every i0) arrives
// in X by 16-byte asynchronous copies issued while the previous node is
// transformed; Y holds the axis-0 exchange.
template <int N0>
__global__ void __launch_bounds__(kS8L*(N0 / kFzColE), 1)
    k_fz_pot2_s8(const float2* __restrict__ XY, float2* __restrict__ pot2G, FzTab tb,
                 const double* __restrict__ knode, const double* __restrict__ invk, int j0, int nb, int first,
                 Geo geo, FzDims d, const float2* __restrict__ tw0, float invN) {
    constexpr int E = kFzColE, T = N0 / E, L = kS8L, NT = L * T;
    constexpr int CPT = 16 * N0 / NT;  // 16-byte copies per thread and node: N0 x 8 d x 2 halves
    static_assert(NT == 2 * N0, "two (r0, c) pairs per thread in the radix-8 stage");
    extern __shared__ float2 fz_sm[];
    float2* X = fz_sm;          // N0 * kS8P
    float2* Y = X + N0 * kS8P;  // N0 * L
    float* sq = reinterpret_cast<float*>(Y + N0 * L);
    float* siq = sq + N0 * L;
    float* sik = siq + N0 * L;
    float* sk2 = sik + nb;
    int a0, q;
    bool nyq;
    fz8_tile(d, blockIdx.x, a0, q, nyq);
    // copy idx = tid + NT i: half h = idx & 1 of the 32-byte piece of (r0, d) = (idx >> 4, (idx >> 1) & 7),
    // from plane row 32 d + a0 (main: columns 4 q .. 4 q + 3; Nyquist: a0 .. a0 + 3) to X[r0][4 d + 2 h];
    // h and d are the same for all of a thread's copies, r0 steps by NT / 16
    const int ch = threadIdx.x & 1, cd = (threadIdx.x >> 1) & 7, cr = threadIdx.x >> 4;
    const long long cstep = (long long)(NT / 16) * (nyq ? d.n1 : (long long)d.n1 * d.H);
    const long long cbase = nyq ? d.nyq + (long long)cr * d.n1 + 32 * cd + a0 + 2 * ch
                                : ((long long)cr * d.n1 + 32 * cd + a0) * d.H + 4 * q + 2 * ch;
    float2* const cdst = X + cr * kS8P + 4 * cd + 2 * ch;
    auto issue = [&](int jj) {
        const float2* src = XY + (long long)jj * d.plane + cbase;
#pragma unroll
        for (int i = 0; i < CPT; ++i) cp_async16(cdst + i * (NT / 16) * kS8P, src + i * cstep);
        cp_async_commit();
    };
    issue(0);
    for (int i = threadIdx.x; i < nb; i += NT) {
        const double k = knode[j0 + i];
        sik[i] = (float)invk[j0 + i];
        sk2[i] = (float)(k * k);
    }
    const int l = threadIdx.x % L, t = threadIdx.x / L;
    const int b = l >> 2, c = l & 3;
    // output line l = 4 b + c: k1 = a + 32 b, k2 = 4 q + c (a = a0), or a = a0 + c and k2 = H
    const int k1 = (nyq ? a0 + c : a0) + 32 * b, k2 = nyq ? d.H : 4 * q + c;
    const long long gbase = (long long)k1 * (d.H + 1) + k2, gstride = (long long)d.n1 * (d.H + 1);
    float2 acc[E];
    float qmin = INFINITY;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k0 = t + T * e;
        const int s = k0 * L + l;
        const float q2 = gsq_f(geo, k0, k1, k2);
        sq[s] = sqrtf(q2);
        siq[s] = q2 > 0.0f ? 1.0f / q2 : 0.0f;
        qmin = fminf(qmin, sqrtf(q2));
        acc[e] = first ? make_float2(0.0f, 0.0f) : pot2G[gbase + k0 * gstride];
    }
    qmin = fz_warp_min(qmin);
    const bool g0 = (t == 0 && k1 == 0 && k2 == 0);
    const float2 acc00 = acc[0];
    const int pc = threadIdx.x & 3;
    for (int jj = 0; jj < nb; ++jj) {
        cp_async_wait_all();
        __syncthreads();  // X holds node jj (the first time also: the node and |G| tables are staged)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r0 = (threadIdx.x + NT * h) >> 2;
            float2 u[8];
#pragma unroll
            for (int m = 0; m < 8; ++m) u[m] = X[r0 * kS8P + 4 * m + pc];
            fz::dft8<-1>(u);
#pragma unroll
            for (int m = 0; m < 8; ++m) X[r0 * kS8P + 4 * m + pc] = u[m];
        }
        __syncthreads();
        float2 v[E];
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = X[(t + T * e) * kS8P + l];
        __syncthreads();  // X is read: the next node's copies may land
        if (jj + 1 < nb) issue(jj + 1);
        // Y is free: the previous node's axis-0 reads of Y came before this node's barriers
        // (twiddles from the table: register twiddles would spill beside the accumulators)
        fz::line_fft<N0, E, -1>(v, Y + l, S8ColIdx(), t, tw0);
        const float ik = sik[jj], kj2 = sk2[jj];
        float f[E];
        auto factors = [&](auto near) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int s = (t + T * e) * L + l;
                f[e] = fz_node_kernel<false, decltype(near)::value>(tb, sq[s], ik, siq[s], kj2) * invN;
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
    }
    if (g0) acc[0] = acc00;
#pragma unroll
    for (int e = 0; e < E; ++e) pot2G[gbase + (t + T * e) * gstride] = acc[e];
}

}  // namespace
