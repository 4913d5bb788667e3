// Smooth-PME building blocks shared by the local pseudopotential and Ewald:
// cardinal B-spline charge spreading and the gradient gather for forces
// (src/dftpy/ewald.py:63-82, :137-194, :810-864; pseudo/__init__.py:523-571).
#pragma once
#include "common.cuh"

namespace ofdft {

constexpr int kMaxOrder = 16;

// out[n] = M_order(x + n - 1), n = 1..order; out[0] = 0 (ewald.py:63-82)
__device__ inline void bspline_mn_dev(double x, int order, double* Mn) {
    for (int i = 0; i <= order; ++i) Mn[i] = 0.0;
    Mn[1] = x;
    Mn[2] = 1.0 - x;
    for (int i = 3; i <= order; ++i) {
        for (int j = 0; j < i; ++j) {
            int n = i - j;
            Mn[n] = (x + n - 1) * Mn[n] + (j + 1 - x) * Mn[n - 1];
            Mn[n] /= (double)(i - 1);
        }
    }
}

__device__ inline int pmod(long long a, int n) {
    long long r = a % n;
    return (int)(r < 0 ? r + n : r);
}

// One block per atom: Q[l0(i), l1(j), l2(k)] += w_a M(i) M(j) M(k) with
// l_d(i) = (1 + floor(u_d) - i) mod n_d, u = frac * n (ewald.py:172-194).
// frac: natoms x 3 fractional coordinates in [0, 1).
template <typename T>
__global__ void k_pme_spread(const double* __restrict__ frac, const double* __restrict__ w, const int* __restrict__ sel,
                             int order, Geo geo, T* Q) {
    __shared__ double M[3][kMaxOrder + 1];
    __shared__ int base[3];
    const int a = sel ? sel[blockIdx.x] : blockIdx.x;
    if (threadIdx.x < 3) {
        const int d = threadIdx.x;
        const int n = d == 0 ? geo.n0 : (d == 1 ? geo.n1 : geo.n2);
        double up = frac[3 * a + d] * (double)n;
        double fl = floor(up);
        bspline_mn_dev(up - fl, order, M[d]);
        base[d] = (int)fl;
    }
    __syncthreads();
    const double wa = w ? w[a] : 1.0;
    const int o3 = order * order * order;
    for (int t = threadIdx.x; t < o3; t += blockDim.x) {
        int i = t / (order * order), j = (t / order) % order, k = t % order;
        int l0 = pmod(1LL + base[0] - i, geo.n0);
        int l1 = pmod(1LL + base[1] - j, geo.n1);
        int l2 = pmod(1LL + base[2] - k, geo.n2);
        double v = wa * M[0][i + 1] * M[1][j + 1] * M[2][k + 1];
        atomicAdd(&Q[((long long)l0 * geo.n1 + l1) * geo.n2 + l2], (T)v);
    }
}

// One block per atom: g_a = sum_{ijk} (dQ/du . cinv) * field[l(ijk)], the PME
// gradient of _ForcePME / Forces_rec_PME with dQ_d = n_d dM_d (M_{order-1}
// differences) times the other two M_order factors.  out[3a+c] = scale_a * g_c.
template <typename T>
__global__ void k_pme_gather(const double* __restrict__ frac, const int* __restrict__ sel, int order, Geo geo,
                             const T* __restrict__ field, const double* __restrict__ cinv,
                             const double* __restrict__ scale, double* out) {
    __shared__ double M[3][kMaxOrder + 1];
    __shared__ double dM[3][kMaxOrder + 1];
    __shared__ int base[3];
    __shared__ double red[3][RED_THREADS / 32];
    const int a = sel ? sel[blockIdx.x] : blockIdx.x;
    if (threadIdx.x < 3) {
        const int d = threadIdx.x;
        const int n = d == 0 ? geo.n0 : (d == 1 ? geo.n1 : geo.n2);
        double up = frac[3 * a + d] * (double)n;
        double fl = floor(up);
        double M2[kMaxOrder + 1];
        bspline_mn_dev(up - fl, order, M[d]);
        bspline_mn_dev(up - fl, order - 1, M2);
        M2[order] = 0.0;
        for (int i = 0; i < order; ++i) dM[d][i] = (double)n * (M2[i + 1] - M2[i]);
        base[d] = (int)fl;
    }
    __syncthreads();
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    const int o3 = order * order * order;
    for (int t = threadIdx.x; t < o3; t += blockDim.x) {
        int i = t / (order * order), j = (t / order) % order, k = t % order;
        int l0 = pmod(1LL + base[0] - i, geo.n0);
        int l1 = pmod(1LL + base[1] - j, geo.n1);
        int l2 = pmod(1LL + base[2] - k, geo.n2);
        double f = (double)field[((long long)l0 * geo.n1 + l1) * geo.n2 + l2];
        double q0 = dM[0][i] * M[1][j + 1] * M[2][k + 1];
        double q1 = M[0][i + 1] * dM[1][j] * M[2][k + 1];
        double q2 = M[0][i + 1] * M[1][j + 1] * dM[2][k];
        // (dQ . cinv)_c = sum_d dQ_d cinv[d][c]
        g0 += (q0 * cinv[0] + q1 * cinv[3] + q2 * cinv[6]) * f;
        g1 += (q0 * cinv[1] + q1 * cinv[4] + q2 * cinv[7]) * f;
        g2 += (q0 * cinv[2] + q1 * cinv[5] + q2 * cinv[8]) * f;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        g0 += __shfl_down_sync(0xffffffffu, g0, o);
        g1 += __shfl_down_sync(0xffffffffu, g1, o);
        g2 += __shfl_down_sync(0xffffffffu, g2, o);
    }
    if (lane == 0) {
        red[0][wid] = g0;
        red[1][wid] = g1;
        red[2][wid] = g2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0, s1 = 0, s2 = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
            s0 += red[0][w];
            s1 += red[1][w];
            s2 += red[2][w];
        }
        const double sc = scale ? scale[a] : 1.0;
        out[3 * a + 0] = sc * s0;
        out[3 * a + 1] = sc * s1;
        out[3 * a + 2] = sc * s2;
    }
}

// B(G) = bm0(i) bm1(j) bm2(k) from per-axis complex tables (ewald.py:44-55)
__device__ inline void barray(const double* bre, const double* bim, const Geo& g, long long idx, double& br,
                              double& bi) {
    int k = (int)(idx % g.n2h);
    long long t = idx / g.n2h;
    int j = (int)(t % g.n1);
    int i = (int)(t / g.n1);
    // axis offsets in the packed tables: [0, n0), [n0, n0+n1), [n0+n1, ...)
    double ar = bre[i], ai = bim[i];
    double cr = bre[g.n0 + j], ci = bim[g.n0 + j];
    double xr = ar * cr - ai * ci, xi = ar * ci + ai * cr;
    double er = bre[g.n0 + g.n1 + k], ei = bim[g.n0 + g.n1 + k];
    br = xr * er - xi * ei;
    bi = xr * ei + xi * er;
}

}  // namespace ofdft
