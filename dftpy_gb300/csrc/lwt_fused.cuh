// Fused float32 pipeline of the density-dependent (k_F-node) kernel for
// power-of-two grids (each axis 32..256, the contiguous axis 32..512).
//
// It computes what the cuFFT pipeline computes (lwt.py:226-306, kernel.py:379-405):
//   P_j = IFFT(K_j FFT(rho^beta)/N), M_j = IFFT(K'_j/k_j FFT(rho^beta)/N)
//   pot1 (+)= linear interpolation of P over each point's k_F interval
//   pot3 (+)= the same interpolation of M                          (kdd = 3)
//   pot2(G) (+)= sum_j K_j(G) FFT(rho^alpha W_j)(G)/N              (kdd > 1)
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
};

constexpr int kFzLines = 16;  // lines per column tile
constexpr int kFzColE = 16;   // points per thread along a column
constexpr int kFzRowE = 8;    // complex points per thread along a row
constexpr int kFzRowThreads = 256;

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

// X_j, Y_j of a batch of nodes, inverse-transformed along axis 0.
template <int N0>
__global__ void __launch_bounds__(kFzLines * (N0 / kFzColE))
    k_fz_nodes(const float2* __restrict__ rbG, float2* __restrict__ XY, Table<float> tab, Nodes nd, int j0, int nb,
               int mcalc, Geo geo, FzDims d, const float2* __restrict__ tw, double invN) {
    constexpr int E = kFzColE, T = N0 / E;
    extern __shared__ float2 fz_sm[];
    float* sinvk = reinterpret_cast<float*>(fz_sm + fz::col_slots(N0));
    for (int q = threadIdx.x; q < nb; q += blockDim.x) sinvk[q] = (float)nd.invk[j0 + q];
    __syncthreads();
    const int l = threadIdx.x % kFzLines, t = threadIdx.x / kFzLines;
    int k1, k2;
    long long pbase, pstride, gbase, gstride;
    fz_axis0_tile(d, blockIdx.x, l, k1, k2, pbase, pstride, gbase, gstride);
    const float invNt = (float)invN;
    float2 z[E];
    float q[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k0 = t + T * e;
        const float2 a = rbG[gbase + k0 * gstride];
        z[e] = make_float2(a.x * invNt, a.y * invNt);
        q[e] = sqrtf(gsq_f(geo, k0, k1, k2));
    }
    const bool g0 = (t == 0 && k1 == 0 && k2 == 0);  // G = 0 sits in register 0 of thread t = 0
    float2* sm = fz_sm + l;
    for (int jj = 0; jj < nb; ++jj) {
        const float ik = sinvk[jj];
        float2 v[E];
        float kd[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            float K, KD;
            node_kernel<float>(tab, q[e], ik, mcalc != 0, (g0 && e == 0) ? 0 : 1, K, KD);
            v[e] = make_float2(K * z[e].x, K * z[e].y);
            kd[e] = KD * ik;
        }
        __syncthreads();
        fz::line_fft<N0, E, +1>(v, sm, fz::ColIdx(), t, tw);
        float2* outp = XY + (long long)jj * d.plane + pbase;
#pragma unroll
        for (int e = 0; e < E; ++e) outp[(t + T * e) * pstride] = v[e];
        if (mcalc) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = make_float2(kd[e] * z[e].x, kd[e] * z[e].y);
            __syncthreads();
            fz::line_fft<N0, E, +1>(v, sm, fz::ColIdx(), t, tw);
            float2* outm = XY + (long long)(nb + jj) * d.plane + pbase;
#pragma unroll
            for (int e = 0; e < E; ++e) outm[(t + T * e) * pstride] = v[e];
        }
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
        for (int e = 0; e < E; ++e) v[e] = line[(long long)(t + T * e) * d.H];
        fz::line_fft<N1, E, S>(v, fz_sm + l, fz::ColIdx(), t, tw);
#pragma unroll
        for (int e = 0; e < E; ++e) line[(long long)(t + T * e) * d.H] = v[e];
    } else {
        const int t = threadIdx.x % T, l = threadIdx.x / T;
        const int i0 = (tile - tiles_main) * kFzLines + l;
        float2* line = base + d.nyq + (long long)i0 * N1;
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = line[t + T * e];
        fz::line_fft<N1, E, S>(v, fz_sm + l * fz::row_slots(N1), fz::RowIdx(), t, tw);
#pragma unroll
        for (int e = 0; e < E; ++e) line[t + T * e] = v[e];
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
    int m, j0, nb, nplanes, kdd, first;
    double kfclip;
    FzDims d;
    FzTw tw;
};

// per-point interval state for the interpolation (lwt.py:252-306 with the
// float32 closed-interior membership): ir >= 0 interval index with coordinate
// tr; ir = -1 small-k_F branch of node 0 with coordinate tr; ir = -2 nothing.
__device__ __forceinline__ void fz_point_state(double kf, const double* kn, const double* kup, int m, int& ir,
                                               float& tr) {
    const Member mb = membership(kf, kn, kup, m, true);
    if (mb.ilast >= 0) {
        const int i = mb.ilast;
        ir = i;
        tr = (float)(kf - kn[i]) / (float)(kn[i + 1] - kn[i]);
    } else if (mb.small) {
        ir = -1;
        tr = (float)(kf - kn[0]) / (float)kn[0];
    } else {
        ir = -2;
        tr = 0.0f;
    }
}

template <int H>
__device__ __forceinline__ void fz_load_nodes(const FzRowArgs& a, double* kn, double* kup) {
    for (int q = threadIdx.x; q < a.m; q += blockDim.x) {
        kn[q] = a.kn[q];
        kup[q] = a.kup[q];
    }
}

// Axis-2 C2R of every plane of the batch, row by row, with the interpolation
// of the P (and M) values into pot1 (pot3) at every point of the row.
template <int H>
__global__ void __launch_bounds__(kFzRowThreads) k_fz_c2r_rows(FzRowArgs a) {
    constexpr int E = kFzRowE, T = H / E, ROWS = kFzRowThreads / T, P = 2 * E;
    constexpr int RS = fz::row_slots(H);
    extern __shared__ double fz_rsm[];
    double* kn = fz_rsm;
    double* kup = fz_rsm + a.m;
    float2* rows = reinterpret_cast<float2*>(fz_rsm + 2 * a.m);
    fz_load_nodes<H>(a, kn, kup);
    __syncthreads();
    const int t = threadIdx.x % T, l = threadIdx.x / T;
    const long long row = (long long)blockIdx.x * ROWS + l;
    const int n2 = 2 * H;
    float2* sm = rows + l * RS;
    const fz::RowIdx ix;
    int ir[P];
    float tr[P], acc1[P], acc3[P];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int mm = t + T * e;
        const float2 kk = *reinterpret_cast<const float2*>(a.kf + row * n2 + 2 * mm);
        fz_point_state(fmin((double)kk.x, a.kfclip), kn, kup, a.m, ir[2 * e], tr[2 * e]);
        fz_point_state(fmin((double)kk.y, a.kfclip), kn, kup, a.m, ir[2 * e + 1], tr[2 * e + 1]);
    }
#pragma unroll
    for (int q = 0; q < P; ++q) acc1[q] = acc3[q] = 0.0f;
    for (int p = 0; p < a.nplanes; ++p) {
        const bool isM = p >= a.nb;
        const int j = a.j0 + (isM ? p - a.nb : p);
        const float2* src = a.XY + (long long)p * a.d.plane;
        __syncthreads();  // sm free
#pragma unroll
        for (int e = 0; e < E; ++e) sm[ix(t + T * e)] = src[row * H + t + T * e];
        if (t == 0) sm[ix(H)] = src[a.d.nyq + row];
        __syncthreads();
        float2 v[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int k = t + T * e;
            float2 X = sm[ix(k)], Y = sm[ix(H - k)];
            if (k == 0) {
                X.y = 0.0f;
                Y.y = 0.0f;
            }
            // Z = (X + conj Y) + i w^k (X - conj Y), w = exp(+2 pi i/n2)
            const float2 A = make_float2(X.x + Y.x, X.y - Y.y);
            const float2 B = make_float2(X.x - Y.x, X.y + Y.y);
            const float2 wB = fz::cmulc(B, __ldg(a.tw.tr + k));
            v[e] = make_float2(A.x - wB.y, A.y + wB.x);
        }
        __syncthreads();  // every pair read before the transform writes sm
        fz::line_fft<H, E, +1>(v, sm, ix, t, a.tw.th);
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const float val = (q & 1) ? v[q >> 1].y : v[q >> 1].x;
            if (!isM) {
                if (ir[q] >= 0) {
                    if (j == ir[q]) acc1[q] += val * (1.0f - tr[q]);
                    else if (j == ir[q] + 1) acc1[q] += val * tr[q];
                } else if (ir[q] == -1 && j == 0) {
                    acc1[q] += val * tr[q];
                }
            } else if (a.kdd == 3 && ir[q] >= 0) {
                if (j == ir[q]) acc3[q] += val * (1.0f - tr[q]);
                else if (j == ir[q] + 1) acc3[q] += val * tr[q];
            }
        }
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const long long r = row * n2 + 2 * (t + T * e);
        float2 o1 = make_float2(acc1[2 * e], acc1[2 * e + 1]);
        if (!a.first) {
            const float2 old = *reinterpret_cast<const float2*>(a.pot1 + r);
            o1 = make_float2(old.x + o1.x, old.y + o1.y);
        }
        *reinterpret_cast<float2*>(a.pot1 + r) = o1;
        if (a.kdd == 3) {
            float2 o3 = make_float2(acc3[2 * e], acc3[2 * e + 1]);
            if (!a.first) {
                const float2 old = *reinterpret_cast<const float2*>(a.pot3 + r);
                o3 = make_float2(old.x + o3.x, old.y + o3.y);
            }
            *reinterpret_cast<float2*>(a.pot3 + r) = o3;
        }
    }
}

// hat weights of one point (lwt.py:266-296, linear): up to three nodes
// base..base+2 with weights rA*W[d]; the small-k_F weight of node 0 is folded
// into W[0] (node 0 is then always the base).
__device__ __forceinline__ void fz_hat_state(double kf, float rA, const double* kn, const double* kup, int m,
                                             int& base, float (&rw)[3]) {
    const Member mb = membership(kf, kn, kup, m, true);
    const int ints[2] = {mb.ilast, mb.iprev};
    base = mb.ilast >= 0 ? (mb.iprev >= 0 ? mb.iprev : mb.ilast) : 0;
    float W[3] = {0.0f, 0.0f, 0.0f};
    if (mb.ilast >= 0) {
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int i = ints[s];
            if (i < 0) continue;
            const float tt = (float)(kf - kn[i]) / (float)(kn[i + 1] - kn[i]);
            W[i - base] += 1.0f - tt;
            W[i + 1 - base] += tt;
        }
    }
    if (mb.small && base == 0) W[0] += (float)(kf - kn[0]) / (float)kn[0];
#pragma unroll
    for (int s = 0; s < 3; ++s) rw[s] = rA * W[s];
}

// rho^alpha W_j of every node of the batch, R2C along axis 2, row by row.
template <int H>
__global__ void __launch_bounds__(kFzRowThreads) k_fz_r2c_rows(FzRowArgs a) {
    constexpr int E = kFzRowE, T = H / E, ROWS = kFzRowThreads / T, P = 2 * E;
    constexpr int RS = fz::row_slots(H);
    extern __shared__ double fz_rsm[];
    double* kn = fz_rsm;
    double* kup = fz_rsm + a.m;
    float2* rows = reinterpret_cast<float2*>(fz_rsm + 2 * a.m);
    fz_load_nodes<H>(a, kn, kup);
    __syncthreads();
    const int t = threadIdx.x % T, l = threadIdx.x / T;
    const long long row = (long long)blockIdx.x * ROWS + l;
    const int n2 = 2 * H;
    float2* sm = rows + l * RS;
    const fz::RowIdx ix;
    int base[P];
    float rw[P][3];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int mm = t + T * e;
        const float2 kk = *reinterpret_cast<const float2*>(a.kf + row * n2 + 2 * mm);
        const float2 ra = *reinterpret_cast<const float2*>(a.rA + row * n2 + 2 * mm);
        fz_hat_state(fmin((double)kk.x, a.kfclip), ra.x, kn, kup, a.m, base[2 * e], rw[2 * e]);
        fz_hat_state(fmin((double)kk.y, a.kfclip), ra.y, kn, kup, a.m, base[2 * e + 1], rw[2 * e + 1]);
    }
    for (int jj = 0; jj < a.nb; ++jj) {
        const int j = a.j0 + jj;
        float2 v[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            float u[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int q = 2 * e + h;
                const int dd = j - base[q];
                u[h] = dd == 0 ? rw[q][0] : (dd == 1 ? rw[q][1] : (dd == 2 ? rw[q][2] : 0.0f));
            }
            v[e] = make_float2(u[0], u[1]);
        }
        __syncthreads();  // sm free
        fz::line_fft<H, E, -1>(v, sm, ix, t, a.tw.th);
        __syncthreads();  // the transform's last reads done
#pragma unroll
        for (int e = 0; e < E; ++e) sm[ix(t + T * e)] = v[e];
        __syncthreads();
        float2* dst = a.XY + (long long)jj * a.d.plane;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int k = t + T * e;
            const float2 Zk = sm[ix(k)], Zc = sm[ix((H - k) & (H - 1))];
            // X = (Zk + conj Zc)/2 - i w^-k (Zk - conj Zc)/2, w^-k = exp(-2 pi i k/n2)
            const float2 A = make_float2(0.5f * (Zk.x + Zc.x), 0.5f * (Zk.y - Zc.y));
            const float2 B = make_float2(0.5f * (Zk.x - Zc.x), 0.5f * (Zk.y + Zc.y));
            const float2 wB = fz::cmul(B, __ldg(a.tw.tr + k));
            dst[row * H + k] = make_float2(A.x + wB.y, A.y - wB.x);
        }
        if (t == 0) {
            const float2 Z0 = sm[ix(0)];
            dst[a.d.nyq + row] = make_float2(Z0.x - Z0.y, 0.0f);
        }
    }
}

// Axis-0 forward transform of the batch's planes, K_j(G)/N applied and summed
// into pot2(G) (lwt.py:266-296; the sum starts from the previous batches').
template <int N0>
__global__ void __launch_bounds__(kFzLines * (N0 / kFzColE))
    k_fz_pot2(const float2* __restrict__ XY, float2* __restrict__ pot2G, Table<float> tab, Nodes nd, int j0, int nb,
              int first, Geo geo, FzDims d, const float2* __restrict__ tw, double invN) {
    constexpr int E = kFzColE, T = N0 / E;
    extern __shared__ float2 fz_sm[];
    float* sinvk = reinterpret_cast<float*>(fz_sm + fz::col_slots(N0));
    for (int q = threadIdx.x; q < nb; q += blockDim.x) sinvk[q] = (float)nd.invk[j0 + q];
    __syncthreads();
    const int l = threadIdx.x % kFzLines, t = threadIdx.x / kFzLines;
    int k1, k2;
    long long pbase, pstride, gbase, gstride;
    fz_axis0_tile(d, blockIdx.x, l, k1, k2, pbase, pstride, gbase, gstride);
    const float invNt = (float)invN;
    float q[E];
    float2 acc[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k0 = t + T * e;
        q[e] = sqrtf(gsq_f(geo, k0, k1, k2));
        acc[e] = first ? make_float2(0.0f, 0.0f) : pot2G[gbase + k0 * gstride];
    }
    const bool g0 = (t == 0 && k1 == 0 && k2 == 0);
    float2* sm = fz_sm + l;
    for (int jj = 0; jj < nb; ++jj) {
        const float ik = sinvk[jj];
        const float2* inp = XY + (long long)jj * d.plane + pbase;
        float2 v[E];
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = inp[(t + T * e) * pstride];
        __syncthreads();
        fz::line_fft<N0, E, -1>(v, sm, fz::ColIdx(), t, tw);
#pragma unroll
        for (int e = 0; e < E; ++e) {
            float K, KD;
            node_kernel<float>(tab, q[e], ik, false, (g0 && e == 0) ? 0 : 1, K, KD);
            const float f = K * invNt;
            acc[e].x += f * v[e].x;
            acc[e].y += f * v[e].y;
        }
    }
#pragma unroll
    for (int e = 0; e < E; ++e) pot2G[gbase + (t + T * e) * gstride] = acc[e];
}

}  // namespace
