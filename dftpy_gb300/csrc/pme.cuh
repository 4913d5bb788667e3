// Smooth-PME building blocks shared by the local pseudopotential and Ewald:
// cardinal B-spline charge spreading, Q[l0(i), l1(j), l2(k)] += w_a M(i) M(j) M(k)
// with l_d(i) = (1 + floor(u_d) - i) mod n_d, u = frac * n (ewald.py:172-194),
// and the gradient gather for forces (src/dftpy/ewald.py:63-82, :137-194,
// :810-864; pseudo/__init__.py:523-571).
#pragma once
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

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

// ---------------------------------------------------------------------------
// Deterministic spreading.  The grid is cut into 8^3 tiles; the host lists, for
// every tile that some atom's order^3 stencil touches, the atoms (positions in
// the spread list) that touch it, in list order.  One block per touched tile,
// one thread per grid point: the thread sums the contributions of its tile's
// atoms in that order in float64 and stores the point once.  The sum at every
// point therefore has a fixed order and Q is the same bits on every run (a
// per-atom scatter with global atomics sums in arrival order).
constexpr int kPmeTile = 8;

struct PmeTiles {
    int ntiles = 0, nlist = 0, order = 0;
    int* tile = nullptr;   // tile ids (t0 T1 + t1) T2 + t2
    int* start = nullptr;  // ntiles + 1 offsets into atom
    int* atom = nullptr;   // list positions
    int* base = nullptr;   // 3 per list position: floor(u_d)
    double* M = nullptr;   // 3 (order + 1) per list position: M_order(x + n - 1), n = 0..order
};

// Builds the tile lists on the host and uploads them into buffers of sc named
// prefix + "...".  frac: 3 per atom of the whole set (host); list: the atoms to
// spread (host, nullptr = 0..nlist-1).  The stencil base floor(frac n) is the
// same IEEE product and floor the device computes.
inline PmeTiles pme_tiles_build(Scratch& sc, const std::string& prefix, const double* frac, const int* list,
                                int nlist, int order, const int nr[3], cudaStream_t st) {
    PmeTiles t;
    t.nlist = nlist;
    t.order = order;
    if (nlist <= 0) return t;
    int nt[3];
    for (int d = 0; d < 3; ++d) nt[d] = (nr[d] + kPmeTile - 1) / kPmeTile;
    std::vector<long long> key;
    key.reserve((size_t)nlist * 27);
    for (int q = 0; q < nlist; ++q) {
        const int a = list ? list[q] : q;
        std::vector<int> tl[3];
        for (int d = 0; d < 3; ++d) {
            const long long b = (long long)std::floor(frac[3 * (size_t)a + d] * (double)nr[d]);
            for (int i = 0; i < order; ++i) {
                long long l = (1 + b - i) % nr[d];
                if (l < 0) l += nr[d];
                const int tt = (int)(l / kPmeTile);
                if (std::find(tl[d].begin(), tl[d].end(), tt) == tl[d].end()) tl[d].push_back(tt);
            }
        }
        for (int x : tl[0])
            for (int y : tl[1])
                for (int z : tl[2]) key.push_back((((long long)x * nt[1] + y) * nt[2] + z) * nlist + q);
    }
    std::sort(key.begin(), key.end());
    std::vector<int> tile, start, atom(key.size());
    for (size_t p = 0; p < key.size(); ++p) {
        const int tid = (int)(key[p] / nlist);
        atom[p] = (int)(key[p] % nlist);
        if (tile.empty() || tile.back() != tid) {
            tile.push_back(tid);
            start.push_back((int)p);
        }
    }
    start.push_back((int)key.size());
    t.ntiles = (int)tile.size();
    t.tile = (int*)sc.get(prefix + "tile", tile.size() * sizeof(int));
    t.start = (int*)sc.get(prefix + "start", start.size() * sizeof(int));
    t.atom = (int*)sc.get(prefix + "atom", atom.size() * sizeof(int));
    t.base = (int*)sc.get(prefix + "base", 3 * (size_t)nlist * sizeof(int));
    t.M = (double*)sc.get(prefix + "M", 3 * (size_t)(order + 1) * nlist * sizeof(double));
    OFDFT_CK(cudaMemcpyAsync(t.tile, tile.data(), tile.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    OFDFT_CK(cudaMemcpyAsync(t.start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    OFDFT_CK(cudaMemcpyAsync(t.atom, atom.data(), atom.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    // the host vectors die with this call: let the copies finish first
    OFDFT_CK(cudaStreamSynchronize(st));
    return t;
}

// stencil base and B-spline weights of every list position (one thread each)
static __global__ void k_pme_prep(const double* __restrict__ frac, const int* __restrict__ list, int nlist, int order,
                                  Geo geo, int* base, double* M) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nlist) return;
    const int a = list ? list[q] : q;
    for (int d = 0; d < 3; ++d) {
        const int n = d == 0 ? geo.n0 : (d == 1 ? geo.n1 : geo.n2);
        const double up = frac[3 * a + d] * (double)n;
        const double fl = floor(up);
        bspline_mn_dev(up - fl, order, M + (3 * (size_t)q + d) * (order + 1));
        base[3 * q + d] = (int)fl;
    }
}

// Q at every point of a touched tile: sum over the tile's atoms, in list order,
// of w_a M0(i) M1(j) M2(k) with i = (1 + base_0 - l0) mod n0 (< order), etc.
template <typename T>
__global__ void __launch_bounds__(kPmeTile* kPmeTile* kPmeTile)
    k_pme_tiles(PmeTiles t, const double* __restrict__ w, const int* __restrict__ list, Geo geo, T* Q) {
    const int tid = t.tile[blockIdx.x];
    const int T1 = (geo.n1 + kPmeTile - 1) / kPmeTile, T2 = (geo.n2 + kPmeTile - 1) / kPmeTile;
    const int l0 = (tid / (T1 * T2)) * kPmeTile + (threadIdx.x >> 6);
    const int l1 = ((tid / T2) % T1) * kPmeTile + ((threadIdx.x >> 3) & 7);
    const int l2 = (tid % T2) * kPmeTile + (threadIdx.x & 7);
    if (l0 >= geo.n0 || l1 >= geo.n1 || l2 >= geo.n2) return;
    const int order = t.order, o1 = order + 1;
    double v = 0.0;
    for (int p = t.start[blockIdx.x]; p < t.start[blockIdx.x + 1]; ++p) {
        const int q = t.atom[p];
        const int* b = t.base + 3 * q;
        const double* M0 = t.M + (3 * (size_t)q) * o1;
        const double* M1 = M0 + o1;
        const double* M2 = M1 + o1;
        const double wa = w ? w[list ? list[q] : q] : 1.0;
        // n >= order in practice; the loops also cover a stencil that wraps onto itself
        for (int i = pmod(1LL + b[0] - l0, geo.n0); i < order; i += geo.n0)
            for (int j = pmod(1LL + b[1] - l1, geo.n1); j < order; j += geo.n1)
                for (int k = pmod(1LL + b[2] - l2, geo.n2); k < order; k += geo.n2)
                    v += wa * M0[i + 1] * M1[j + 1] * M2[k + 1];
    }
    Q[((long long)l0 * geo.n1 + l1) * geo.n2 + l2] = (T)v;
}

// Q = the spread of the list (Q zeroed here); t from pme_tiles_build with the
// same list and order.  d_frac, d_list, d_w on the device (d_list, d_w may be null).
template <typename T>
void pme_spread(const PmeTiles& t, const double* d_frac, const int* d_list, const double* d_w, const Geo& geo, T* Q,
                size_t qbytes, cudaStream_t st) {
    OFDFT_CK(cudaMemsetAsync(Q, 0, qbytes, st));
    if (t.nlist <= 0 || t.ntiles <= 0) return;
    k_pme_prep<<<(t.nlist + 127) / 128, 128, 0, st>>>(d_frac, d_list, t.nlist, t.order, geo, t.base, t.M);
    OFDFT_LAUNCH_CHECK();
    k_pme_tiles<T><<<t.ntiles, kPmeTile * kPmeTile * kPmeTile, 0, st>>>(t, d_w, d_list, geo, Q);
    OFDFT_LAUNCH_CHECK();
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
