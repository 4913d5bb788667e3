// Persistent batched E+V evaluation of many independent systems.
//
// One cooperative launch evaluates the energy and potential of every system
// of a batch (uneven grids, one precision) for the functionals a batch of
// small systems uses: TF, vW, LDA, Hartree and the local pseudopotential
// (total_functional.py:107-146 with kedf/tf.py, kedf/vw.py,
// xc/semilocal_xc.py:283-341, hartree.py:24-45, pseudo/__init__.py:74-571).
// The reference evaluates one system per call; this path has no counterpart
// there.  The launch walks device work lists of (system, tile) items, stage
// after stage, with a grid-wide barrier between stages:
//   A  rows: the pre-pass per point (TF, LDA, PP energies and potentials,
//      sqrt(rho)), rho + i sqrt(rho) transformed along axis 2 and split into
//      the two half spectra (the R2C of rho and of sqrt(rho));
//   B  columns along axis 1, forward, both half spectra;
//   C  columns along axis 0: forward, 4 pi / G^2 / N (Hartree) and
//      G^2 / 2 / N (vW) applied, inverse;
//   D  columns along axis 1, inverse;
//   E  rows: v_H + i lap assembled from the two half spectra (numpy's irfftn
//      semantics: the imaginary parts of the k2 = 0 and k2 = n2/2 terms are
//      dropped), transformed back along axis 2, and the post-pass per point
//      (vW and Hartree potentials and energies);
//   F  per system: the item partial sums in a fixed order, the energies.
// The transforms are mixed-radix (2, 3, 4, 5, 8) Stockham FFTs in shared
// memory on tiles of `rows` rows or `lines` columns; the block size, rows and
// lines come from an autotuner that times candidate shapes on the batch itself.
// Every sum has a fixed order, so results are bit-stable from run to run.
#include "common.cuh"
#include "pointwise.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

ofdft_grid* e_grid(ofdft_eval* e);
const ofdft_config* e_cfg(const ofdft_eval* e);
const void* e_vloc(const ofdft_eval* e);

using namespace ofdft;
namespace cg = cooperative_groups;

namespace {

constexpr int kPbMaxPass = 8;
constexpr int kPbMaxLen = 128;
constexpr int kPbMaxSys = 128;
constexpr int kPbSumsA = 4;  // TF, XC, PP, N per row item
constexpr int kPbSumsE = 2;  // vW, Hartree per row item

struct PbFft {
    int n, np, tw;  // length, passes, offset of its twiddles exp(-2 pi i k/n), k < n
    int r[kPbMaxPass];
};

template <typename T>
struct PbSys {
    const T* rho;  // per call
    T* V;          // per call
    const T* vloc;
    typename Cplx<T>::type* RG;  // half spectrum of rho, then v_H
    typename Cplx<T>::type* SG;  // half spectrum of sqrt(rho), then lap
    Geo geo;
    int n0, n1, n2, n2h;
    int f0, f1, f2;  // PbFft of each axis
    int tf, vw, xc, h, pp;
    double tf_x, vw_y, dV, invN, ewald;
    int itA, nA, itB, nB, itC, nC;  // first item and item count of each stage
    int ktiles;                     // column tiles per axis-1/axis-0 line set
};

template <typename T>
struct PbArgs {
    PbSys<T>* sys;
    int S;
    const unsigned char* act;
    const PbFft* fft;
    const typename Cplx<T>::type* tw;
    const int* sysA;  // item -> system, row stages
    const int* sysB;  // axis-1 stages
    const int* sysC;  // axis-0 stage
    int nA, nB, nC;
    double* partA;
    double* partE;
    double* E;  // S x OFDFT_NE
    Consts k;
    int rows, lines;
    int bufslots;  // complex slots per exchange buffer
};

// ------------------------------------------------------------ complex math
template <class C>
__device__ __forceinline__ C cadd(C a, C b) {
    return C{a.x + b.x, a.y + b.y};
}
template <class C>
__device__ __forceinline__ C csub(C a, C b) {
    return C{a.x - b.x, a.y - b.y};
}
template <class C>
__device__ __forceinline__ C cmul(C a, C b) {
    return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * conj(b)
template <class C>
__device__ __forceinline__ C cmulc(C a, C b) {
    return C{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
// a * (S i)
template <class C>
__device__ __forceinline__ C mul_si(C a, int S) {
    return S < 0 ? C{a.y, -a.x} : C{-a.y, a.x};
}
template <class C, class R>
__device__ __forceinline__ C cscale(C a, R s) {
    return C{a.x * s, a.y * s};
}

// In-register DFTs of R points, natural order; sign S: -1 forward, +1 inverse
template <int R, class C>
__device__ __forceinline__ void small_dft(C (&u)[R], int S) {
    using F = decltype(u[0].x);
    if constexpr (R == 2) {
        const C a = u[0];
        u[0] = cadd(a, u[1]);
        u[1] = csub(a, u[1]);
    } else if constexpr (R == 3) {
        const F h = (F)0.8660254037844386467637;  // sqrt(3)/2
        const C s = cadd(u[1], u[2]), d = csub(u[1], u[2]);
        const C m = csub(u[0], cscale(s, (F)0.5));
        const C t = mul_si(cscale(d, h), S);
        u[0] = cadd(u[0], s);
        u[1] = cadd(m, t);
        u[2] = csub(m, t);
    } else if constexpr (R == 4) {
        const C a0 = cadd(u[0], u[2]), a1 = csub(u[0], u[2]);
        const C a2 = cadd(u[1], u[3]), a3 = mul_si(csub(u[1], u[3]), S);
        u[0] = cadd(a0, a2);
        u[2] = csub(a0, a2);
        u[1] = cadd(a1, a3);
        u[3] = csub(a1, a3);
    } else if constexpr (R == 5) {
        const F c1 = (F)0.3090169943749474241023, c2 = (F)-0.8090169943749474241023;
        const F s1 = (F)0.9510565162951535721164, s2 = (F)0.5877852522924731291687;
        const C a1 = cadd(u[1], u[4]), b1 = csub(u[1], u[4]);
        const C a2 = cadd(u[2], u[3]), b2 = csub(u[2], u[3]);
        const C r1 = cadd(u[0], cadd(cscale(a1, c1), cscale(a2, c2)));
        const C r2 = cadd(u[0], cadd(cscale(a1, c2), cscale(a2, c1)));
        const C i1 = mul_si(cadd(cscale(b1, s1), cscale(b2, s2)), S);
        const C i2 = mul_si(csub(cscale(b1, s2), cscale(b2, s1)), S);
        u[0] = cadd(u[0], cadd(a1, a2));
        u[1] = cadd(r1, i1);
        u[4] = csub(r1, i1);
        u[2] = cadd(r2, i2);
        u[3] = csub(r2, i2);
    } else {
        static_assert(R == 8, "radix 2, 3, 4, 5 or 8");
        C e[4] = {u[0], u[2], u[4], u[6]}, o[4] = {u[1], u[3], u[5], u[7]};
        small_dft<4>(e, S);
        small_dft<4>(o, S);
        const F h = (F)0.7071067811865475244008;
        const C w1 = cmul(o[1], C{h, S * h});
        const C w2 = mul_si(o[2], S);
        const C w3 = cmul(o[3], C{-h, S * h});
        u[0] = cadd(e[0], o[0]);
        u[4] = csub(e[0], o[0]);
        u[1] = cadd(e[1], w1);
        u[5] = csub(e[1], w1);
        u[2] = cadd(e[2], w2);
        u[6] = csub(e[2], w2);
        u[3] = cadd(e[3], w3);
        u[7] = csub(e[3], w3);
    }
}

// One Stockham pass of radix R over nl lines of n points: element p of line l
// at src/dst[l * ls + p * ps]; the block's threads share the butterflies.
template <int R, class C>
__device__ __forceinline__ void stockham_pass(const C* src, C* dst, int nl, int ls, int ps, int n, int Ns,
                                              const C* __restrict__ tw, int S) {
    const int m = n / R;
    const int step = n / (Ns * R);
    for (int b = threadIdx.x; b < nl * m; b += blockDim.x) {
        const int l = b / m, j = b - l * m;
        const int k = j % Ns;
        C u[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            C x = src[l * ls + (j + q * m) * ps];
            if (q > 0 && Ns > 1) {
                const C w = __ldg(tw + k * q * step);
                x = S < 0 ? cmul(x, w) : cmulc(x, w);
            }
            u[q] = x;
        }
        small_dft<R>(u, S);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int q = 0; q < R; ++q) dst[l * ls + (base + q * Ns) * ps] = u[q];
    }
}

// Transform nl lines (input in b0); returns the buffer that holds the output.
// Entry: b0 written and visible (the caller synchronised); exit: the output
// visible to every thread.
template <class C>
__device__ C* tile_fft(C* b0, C* b1, int nl, int ls, int ps, const PbFft& f, const C* __restrict__ tw, int S) {
    C* src = b0;
    C* dst = b1;
    int Ns = 1;
    for (int p = 0; p < f.np; ++p) {
        const int r = f.r[p];
        switch (r) {
            case 2: stockham_pass<2>(src, dst, nl, ls, ps, f.n, Ns, tw, S); break;
            case 3: stockham_pass<3>(src, dst, nl, ls, ps, f.n, Ns, tw, S); break;
            case 4: stockham_pass<4>(src, dst, nl, ls, ps, f.n, Ns, tw, S); break;
            case 5: stockham_pass<5>(src, dst, nl, ls, ps, f.n, Ns, tw, S); break;
            default: stockham_pass<8>(src, dst, nl, ls, ps, f.n, Ns, tw, S); break;
        }
        __syncthreads();
        C* t = src;
        src = dst;
        dst = t;
        Ns *= r;
    }
    return src;
}

// The same transform with the length known at compile time: the radices, the
// butterfly counts and the index divisions become constants.  The batching
// workload's lengths (and the usual small ones) take this path.
struct RadixList {
    int np;
    int r[kPbMaxPass];
};
__host__ __device__ constexpr RadixList radix_list(int n) {
    RadixList L{0, {0, 0, 0, 0, 0, 0, 0, 0}};
    int m = n;
    while (m % 8 == 0) {
        L.r[L.np++] = 8;
        m /= 8;
    }
    if (m % 4 == 0) {
        L.r[L.np++] = 4;
        m /= 4;
    } else if (m % 2 == 0) {
        L.r[L.np++] = 2;
        m /= 2;
    }
    while (m % 3 == 0) {
        L.r[L.np++] = 3;
        m /= 3;
    }
    while (m % 5 == 0) {
        L.r[L.np++] = 5;
        m /= 5;
    }
    return L;
}
__host__ __device__ constexpr int ns_before(int n, int p) {
    int ns = 1;
    for (int i = 0; i < p; ++i) ns *= radix_list(n).r[i];
    return ns;
}

template <int N, int P, class C>
__device__ __forceinline__ C* ct_passes(C* src, C* dst, int nl, int ls, int ps, const C* __restrict__ tw, int S) {
    constexpr RadixList L = radix_list(N);
    if constexpr (P == L.np) {
        return src;
    } else {
        constexpr int R = L.r[P], NS = ns_before(N, P), M = N / R, STEP = N / (NS * R);
        for (int b = threadIdx.x; b < nl * M; b += blockDim.x) {
            const int l = b / M, j = b - l * M;
            const int k = j % NS;
            C u[R];
#pragma unroll
            for (int q = 0; q < R; ++q) {
                C x = src[l * ls + (j + q * M) * ps];
                if (NS > 1 && q > 0) {
                    const C w = __ldg(tw + k * q * STEP);
                    x = S < 0 ? cmul(x, w) : cmulc(x, w);
                }
                u[q] = x;
            }
            small_dft<R>(u, S);
            const int base = (j / NS) * NS * R + k;
#pragma unroll
            for (int q = 0; q < R; ++q) dst[l * ls + (base + q * NS) * ps] = u[q];
        }
        __syncthreads();
        return ct_passes<N, P + 1>(dst, src, nl, ls, ps, tw, S);
    }
}

template <int N, class C>
__device__ __noinline__ C* tile_fft_ct(C* b0, C* b1, int nl, int ls, int ps, const C* __restrict__ tw, int S) {
    return ct_passes<N, 0>(b0, b1, nl, ls, ps, tw, S);
}

// compile-time lengths where available, else the runtime radix list
template <class C>
__device__ C* tile_fft_any(C* b0, C* b1, int nl, int ls, int ps, const PbFft& f, const C* __restrict__ tw, int S) {
    switch (f.n) {
        case 16: return tile_fft_ct<16>(b0, b1, nl, ls, ps, tw, S);
        case 20: return tile_fft_ct<20>(b0, b1, nl, ls, ps, tw, S);
        case 24: return tile_fft_ct<24>(b0, b1, nl, ls, ps, tw, S);
        case 30: return tile_fft_ct<30>(b0, b1, nl, ls, ps, tw, S);
        case 32: return tile_fft_ct<32>(b0, b1, nl, ls, ps, tw, S);
        case 36: return tile_fft_ct<36>(b0, b1, nl, ls, ps, tw, S);
        case 40: return tile_fft_ct<40>(b0, b1, nl, ls, ps, tw, S);
        case 48: return tile_fft_ct<48>(b0, b1, nl, ls, ps, tw, S);
        case 60: return tile_fft_ct<60>(b0, b1, nl, ls, ps, tw, S);
        case 64: return tile_fft_ct<64>(b0, b1, nl, ls, ps, tw, S);
        case 72: return tile_fft_ct<72>(b0, b1, nl, ls, ps, tw, S);
        case 80: return tile_fft_ct<80>(b0, b1, nl, ls, ps, tw, S);
        case 96: return tile_fft_ct<96>(b0, b1, nl, ls, ps, tw, S);
        case 120: return tile_fft_ct<120>(b0, b1, nl, ls, ps, tw, S);
        case 128: return tile_fft_ct<128>(b0, b1, nl, ls, ps, tw, S);
        default: return tile_fft(b0, b1, nl, ls, ps, f, tw, S);
    }
}

// ------------------------------------------------------------------ stages
// A: pre-pass and the forward row transforms of rows [row0, row0 + rows)
template <typename T>
__device__ void pb_rows_fwd(const PbArgs<T>& a, int item, typename Cplx<T>::type* b0,
                            typename Cplx<T>::type* b1) {
    using C = typename Cplx<T>::type;
    using M = T;
    const int s = a.sysA[item];
    if (!a.act[s]) return;
    const PbSys<T>& y = a.sys[s];
    const long long nrows = (long long)y.n0 * y.n1;
    const long long row0 = (long long)(item - y.itA) * a.rows;
    const int nl = (int)(nrows - row0 < a.rows ? nrows - row0 : a.rows);
    const int n2 = y.n2, ls = n2 + 1;
    const M cTF_E = (M)a.k.cTF_E, cTF_V = (M)a.k.cTF_V, tf_x = (M)y.tf_x, tiny = (M)1e-30;
    const LdaC<M> lc(a.k);
    RunSum<M> sum[kPbSumsA];
    const bool fft = y.h || y.vw;
    for (int e = threadIdx.x; e < nl * n2; e += blockDim.x) {
        const int l = e / n2, p = e - l * n2;
        const long long i = (row0 + l) * n2 + p;
        const M r = y.rho[i];
        M v = (M)0;
        sum[3].add(r);
        if (y.tf) {
            // PowerInt(rho, 5, 3): repeated products then cbrt (math_utils.py:158-176)
            M r5 = r * r;
            r5 *= r;
            r5 *= r;
            r5 *= r;
            sum[0].add(mcbrt(r5) * cTF_E);
            v += cTF_V * mcbrt(r * r) * tf_x;
        }
        if (y.xc) {
            M ex, vx;
            lda_point(r, lc, ex, vx);
            sum[1].add(ex * r);
            v += vx;
        }
        if (y.pp) {
            const M vl = y.vloc[i];
            sum[2].add(vl * r);
            v += vl;
        }
        y.V[i] = v;
        if (fft) b0[l * ls + p] = C{r, msqrt(r > (M)0 ? r : tiny)};  // kedf/vw.py:34-44
    }
    if (fft) {
        __syncthreads();
        const C* z = tile_fft_any(b0, b1, nl, ls, 1, a.fft[y.f2], a.tw + a.fft[y.f2].tw, -1);
        const M half = (M)0.5;
        for (int e = threadIdx.x; e < nl * y.n2h; e += blockDim.x) {
            const int l = e / y.n2h, k = e - l * y.n2h;
            const C Z = z[l * ls + k];
            const C Zc = z[l * ls + (k == 0 ? 0 : n2 - k)];
            const long long o = (row0 + l) * y.n2h + k;
            if (y.h) y.RG[o] = C{(Z.x + Zc.x) * half, (Z.y - Zc.y) * half};
            if (y.vw) y.SG[o] = C{(Z.y + Zc.y) * half, (Zc.x - Z.x) * half};
        }
    }
    double acc[kPbSumsA] = {sum[0].get(), sum[1].get(), sum[2].get(), sum[3].get()};
    block_sum_store_at<kPbSumsA>(acc, a.partA, item);
    __syncthreads();
}

// B / D: columns along axis 1 at (i0, a tile of `lines` consecutive k2)
template <typename T>
__device__ void pb_axis1(const PbArgs<T>& a, int item, int S, typename Cplx<T>::type* b0,
                         typename Cplx<T>::type* b1) {
    using C = typename Cplx<T>::type;
    const int s = a.sysB[item];
    if (!a.act[s]) return;
    const PbSys<T>& y = a.sys[s];
    const int L = a.lines, ps = L + 1;
    const int t = item - y.itB;
    const int i0 = t / y.ktiles, k2a = (t % y.ktiles) * L;
    const int nl = y.n2h - k2a < L ? y.n2h - k2a : L;
    const PbFft& f = a.fft[y.f1];
    for (int w = 0; w < 2; ++w) {
        C* A = w == 0 ? (y.h ? y.RG : nullptr) : (y.vw ? y.SG : nullptr);
        if (!A) continue;
        for (int e = threadIdx.x; e < y.n1 * nl; e += blockDim.x) {
            const int p = e / nl, l = e - p * nl;
            b0[p * ps + l] = A[((long long)i0 * y.n1 + p) * y.n2h + k2a + l];
        }
        __syncthreads();
        const C* z = tile_fft_any(b0, b1, nl, 1, ps, f, a.tw + f.tw, S);
        for (int e = threadIdx.x; e < y.n1 * nl; e += blockDim.x) {
            const int p = e / nl, l = e - p * nl;
            A[((long long)i0 * y.n1 + p) * y.n2h + k2a + l] = z[p * ps + l];
        }
        __syncthreads();
    }
}

// C: columns along axis 0 at (k1, a tile of k2): forward, the G-space factor, inverse
template <typename T>
__device__ void pb_axis0(const PbArgs<T>& a, int item, typename Cplx<T>::type* b0, typename Cplx<T>::type* b1) {
    using C = typename Cplx<T>::type;
    using M = T;
    const int s = a.sysC[item];
    if (!a.act[s]) return;
    const PbSys<T>& y = a.sys[s];
    const int L = a.lines, ps = L + 1;
    const int t = item - y.itC;
    const int k1 = t / y.ktiles, k2a = (t % y.ktiles) * L;
    const int nl = y.n2h - k2a < L ? y.n2h - k2a : L;
    const PbFft& f = a.fft[y.f0];
    const M invN = (M)y.invN, fourpi = (M)(4.0 * M_PI), half = (M)0.5;
    for (int w = 0; w < 2; ++w) {
        C* A = w == 0 ? (y.h ? y.RG : nullptr) : (y.vw ? y.SG : nullptr);
        if (!A) continue;
        for (int e = threadIdx.x; e < y.n0 * nl; e += blockDim.x) {
            const int p = e / nl, l = e - p * nl;
            b0[p * ps + l] = A[((long long)p * y.n1 + k1) * y.n2h + k2a + l];
        }
        __syncthreads();
        C* z = tile_fft_any(b0, b1, nl, 1, ps, f, a.tw + f.tw, -1);
        // G-space factors as the single-system G-space pass applies them
        for (int e = threadIdx.x; e < y.n0 * nl; e += blockDim.x) {
            const int p = e / nl, l = e - p * nl;
            const long long idx = ((long long)p * y.n1 + k1) * y.n2h + k2a + l;
            const M gg = gsq_t<M>(y.geo, idx);
            M fac;
            if (w == 0) fac = (idx == 0) ? (M)0 : fourpi / gg * invN;  // hartree.py:33-35
            else fac = half * gg * invN;                               // vw.py:45-51
            C v = z[p * ps + l];
            v.x = v.x * fac;
            v.y = v.y * fac;
            z[p * ps + l] = v;
        }
        __syncthreads();
        C* other = z == b0 ? b1 : b0;
        const C* u = tile_fft_any(z, other, nl, 1, ps, f, a.tw + f.tw, +1);
        for (int e = threadIdx.x; e < y.n0 * nl; e += blockDim.x) {
            const int p = e / nl, l = e - p * nl;
            A[((long long)p * y.n1 + k1) * y.n2h + k2a + l] = u[p * ps + l];
        }
        __syncthreads();
    }
}

// E: inverse row transforms of v_H + i lap and the post-pass
template <typename T>
__device__ void pb_rows_inv(const PbArgs<T>& a, int item, typename Cplx<T>::type* b0,
                            typename Cplx<T>::type* b1) {
    using C = typename Cplx<T>::type;
    using M = T;
    const int s = a.sysA[item];
    if (!a.act[s]) return;
    const PbSys<T>& y = a.sys[s];
    const long long nrows = (long long)y.n0 * y.n1;
    const long long row0 = (long long)(item - y.itA) * a.rows;
    const int nl = (int)(nrows - row0 < a.rows ? nrows - row0 : a.rows);
    const int n2 = y.n2, ls = n2 + 1;
    RunSum<M> sum[kPbSumsE];
    if (y.h || y.vw) {
        for (int e = threadIdx.x; e < nl * n2; e += blockDim.x) {
            const int l = e / n2, p = e - l * n2;
            const bool upper = p >= y.n2h;
            const int k = upper ? n2 - p : p;
            const long long o = (row0 + l) * y.n2h + k;
            C H = y.h ? y.RG[o] : C{(M)0, (M)0};
            C W = y.vw ? y.SG[o] : C{(M)0, (M)0};
            if (k == 0 || 2 * k == n2) {  // irfftn drops these imaginary parts
                H.y = (M)0;
                W.y = (M)0;
            }
            b0[l * ls + p] = upper ? C{H.x + W.y, W.x - H.y} : C{H.x - W.y, H.y + W.x};
        }
        __syncthreads();
        const C* z = tile_fft_any(b0, b1, nl, ls, 1, a.fft[y.f2], a.tw + a.fft[y.f2].tw, +1);
        const M tiny = (M)1e-30, vw_y = (M)y.vw_y;
        for (int e = threadIdx.x; e < nl * n2; e += blockDim.x) {
            const int l = e / n2, p = e - l * n2;
            const long long i = (row0 + l) * n2 + p;
            const M r = y.rho[i];
            M v = y.V[i];
            const C zz = z[l * ls + p];
            if (y.vw) {
                M sq = msqrt(r > (M)0 ? r : tiny);
                if (fabs(sq) < tiny) sq = tiny;
                const M pw = zz.y / sq;
                if (r > (M)0) sum[0].add(r * pw);
                v += pw * vw_y;
            }
            if (y.h) {
                const M vh = zz.x;
                sum[1].add(vh * r);
                v += vh;
            }
            y.V[i] = v;
        }
    }
    double acc[kPbSumsE] = {sum[0].get(), sum[1].get()};
    block_sum_store_at<kPbSumsE>(acc, a.partE, item);
    __syncthreads();
}

// F: the system's item sums in a fixed order, then its energies
template <typename T>
__device__ void pb_final(const PbArgs<T>& a, int s) {
    if (!a.act[s]) return;
    const PbSys<T>& y = a.sys[s];
    double acc[kPbSumsA + kPbSumsE];
    for (int q = 0; q < kPbSumsA + kPbSumsE; ++q) acc[q] = 0.0;
    for (int it = threadIdx.x; it < y.nA; it += blockDim.x) {
#pragma unroll
        for (int q = 0; q < kPbSumsA; ++q) acc[q] += a.partA[(long long)(y.itA + it) * kPbSumsA + q];
#pragma unroll
        for (int q = 0; q < kPbSumsE; ++q) acc[kPbSumsA + q] += a.partE[(long long)(y.itA + it) * kPbSumsE + q];
    }
    __shared__ double tot[kPbSumsA + kPbSumsE];
    block_sum_store_at<kPbSumsA + kPbSumsE>(acc, tot, 0);
    __syncthreads();
    if (threadIdx.x == 0) {
        double* E = a.E + (long long)s * OFDFT_NE;
        for (int q = 0; q < OFDFT_NE; ++q) E[q] = 0.0;
        const double dV = y.dV;
        E[OFDFT_E_TF] = y.tf ? tot[0] * dV * y.tf_x : 0.0;
        E[OFDFT_E_XC] = y.xc ? tot[1] * dV : 0.0;
        E[OFDFT_E_PP] = y.pp ? tot[2] * dV : 0.0;
        E[OFDFT_E_NELEC] = tot[3] * dV;
        E[OFDFT_E_VW] = y.vw ? tot[4] * dV * y.vw_y : 0.0;
        E[OFDFT_E_H] = y.h ? tot[5] * dV / 2.0 : 0.0;
        E[OFDFT_E_II] = y.ewald;
        // the single-system evaluator's sum, zeros of the absent terms included
        E[OFDFT_E_TOTAL] = E[OFDFT_E_TF] + E[OFDFT_E_VW] + E[OFDFT_E_NL] + E[OFDFT_E_XC] + E[OFDFT_E_H] +
                           E[OFDFT_E_PP] + E[OFDFT_E_II] + E[OFDFT_E_GGA] + E[OFDFT_E_EXT] + E[OFDFT_E_DTTF];
    }
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(256) k_pb_eval(PbArgs<T> a) {
    using C = typename Cplx<T>::type;
    extern __shared__ __align__(16) unsigned char pb_smem[];
    C* b0 = reinterpret_cast<C*>(pb_smem);
    C* b1 = b0 + a.bufslots;
    cg::grid_group grid = cg::this_grid();
    for (int it = blockIdx.x; it < a.nA; it += gridDim.x) pb_rows_fwd(a, it, b0, b1);
    grid.sync();
    for (int it = blockIdx.x; it < a.nB; it += gridDim.x) pb_axis1(a, it, -1, b0, b1);
    grid.sync();
    for (int it = blockIdx.x; it < a.nC; it += gridDim.x) pb_axis0(a, it, b0, b1);
    grid.sync();
    for (int it = blockIdx.x; it < a.nB; it += gridDim.x) pb_axis1(a, it, +1, b0, b1);
    grid.sync();
    for (int it = blockIdx.x; it < a.nA; it += gridDim.x) pb_rows_inv(a, it, b0, b1);
    grid.sync();
    for (int s = blockIdx.x; s < a.S; s += gridDim.x) pb_final(a, s);
}

// ------------------------------------------------------------------- host
// Radices of an FFT length: 8s, then one 4 or 2, then 3s and 5s; false when n
// has another prime factor or is out of range.
bool factorise(int n, PbFft& f) {
    f.n = n;
    f.np = 0;
    f.tw = 0;
    if (n < 2 || n > kPbMaxLen) return false;
    int m = n;
    auto push = [&](int r) {
        if (f.np == kPbMaxPass) return false;
        f.r[f.np++] = r;
        m /= r;
        return true;
    };
    while (m % 8 == 0)
        if (!push(8)) return false;
    if (m % 4 == 0) {
        if (!push(4)) return false;
    } else if (m % 2 == 0) {
        if (!push(2)) return false;
    }
    while (m % 3 == 0)
        if (!push(3)) return false;
    while (m % 5 == 0)
        if (!push(5)) return false;
    return m == 1;
}

struct PbShape {
    int block = 256, rows = 4, lines = 16;
    double ms = 0.0;  // tuned time of one run (0: not timed)
};

// tuned shapes by batch signature (precision and grid sizes), for the process
std::map<std::string, PbShape>& tuned_shapes() {
    static std::map<std::string, PbShape> m;
    return m;
}

}  // namespace

struct ofdft_batch_eval {
    int S = 0, prec = OFDFT_F64;
    std::vector<ofdft_eval*> evs;
    std::vector<PbFft> fft;
    void* d_sys = nullptr;  // PbSys<T>[S]
    std::vector<unsigned char> h_sys;
    PbFft* d_fft = nullptr;
    void* d_tw = nullptr;
    int *d_sysA = nullptr, *d_sysB = nullptr, *d_sysC = nullptr;
    int nA = 0, nB = 0, nC = 0;
    int bufslots = 0;  // complex slots per shared-memory exchange buffer
    double *d_partA = nullptr, *d_partE = nullptr, *d_E = nullptr, *h_E = nullptr;
    unsigned char *d_act = nullptr, *h_act = nullptr;
    PbShape shape;
    int grid = 0;
    size_t smem = 0;
    double tuned_ms = 0.0;
    std::string sig;
    Scratch sc;
    // field sets of the batched optimiser: a descriptor array per (rho, V)
    // pointer set and the evaluation captured once as a CUDA graph (the active
    // mask upload, the cooperative launch, the energies' copy back), replayed
    // on a stream of its own forked from and joined back to the caller's
    struct FieldSet {
        std::vector<void*> key;
        void* d_sys = nullptr;
        cudaGraphExec_t exec = nullptr;
        bool graph_failed = false;
    };
    std::vector<FieldSet> sets;
    cudaStream_t gst = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    ~ofdft_batch_eval() {
        for (FieldSet& f : sets) {
            if (f.exec) cudaGraphExecDestroy(f.exec);
            cudaFree(f.d_sys);
        }
        if (gst) cudaStreamDestroy(gst);
        if (fork_ev) cudaEventDestroy(fork_ev);
        if (join_ev) cudaEventDestroy(join_ev);
        cudaFree(d_sys);
        cudaFree(d_fft);
        cudaFree(d_tw);
        cudaFree(d_sysA);
        cudaFree(d_sysB);
        cudaFree(d_sysC);
        cudaFree(d_partA);
        cudaFree(d_partE);
        cudaFree(d_E);
        cudaFree(d_act);
        cudaFreeHost(h_E);
        cudaFreeHost(h_act);
    }
};

namespace {

bool eligible(ofdft_eval* e, std::string* why) {
    const ofdft_config& c = *e_cfg(e);
    ofdft_grid* g = e_grid(e);
    auto no = [&](const char* m) {
        if (why) *why = m;
        return false;
    };
    if (c.kedf_terms & ~(OFDFT_KE_TF | OFDFT_KE_VW)) return no("kinetic terms other than TF and vW");
    if (c.wte) return no("WTE");
    if (c.vw_sigma > 0.0) return no("vW smoothing");
    if (c.external) return no("external potential");
    if (c.pseudo && !e_vloc(e)) return no("pseudo enabled without v_loc");
    PbFft f;
    for (int d = 0; d < 3; ++d)
        if (!factorise(g->nr[d], f)) return no("an axis length is not a product of 2, 3 and 5 up to 128");
    return true;
}

template <typename T>
void build_t(ofdft_batch_eval* b) {
    using C = typename Cplx<T>::type;
    const int S = b->S;
    // distinct axis lengths and their twiddles
    std::map<int, int> fidx;
    std::vector<C> tw;
    auto fft_of = [&](int n) {
        auto it = fidx.find(n);
        if (it != fidx.end()) return it->second;
        PbFft f;
        factorise(n, f);
        f.tw = (int)tw.size();
        for (int k = 0; k < n; ++k) {
            const double a = -2.0 * M_PI * (double)k / (double)n;
            tw.push_back(C{(T)std::cos(a), (T)std::sin(a)});
        }
        const int id = (int)b->fft.size();
        b->fft.push_back(f);
        fidx[n] = id;
        return id;
    };
    std::vector<PbSys<T>> sys(S);
    std::vector<int> sysA, sysB, sysC;
    const int L = b->shape.lines, R = b->shape.rows;
    for (int s = 0; s < S; ++s) {
        ofdft_eval* e = b->evs[s];
        ofdft_grid* g = e_grid(e);
        const ofdft_config& c = *e_cfg(e);
        PbSys<T>& y = sys[s];
        memset(&y, 0, sizeof(y));
        y.n0 = g->nr[0];
        y.n1 = g->nr[1];
        y.n2 = g->nr[2];
        y.n2h = g->n2h;
        y.geo = g->geo;
        y.f0 = fft_of(y.n0);
        y.f1 = fft_of(y.n1);
        y.f2 = fft_of(y.n2);
        y.tf = (c.kedf_terms & OFDFT_KE_TF) != 0;
        y.vw = (c.kedf_terms & OFDFT_KE_VW) != 0;
        y.xc = c.xc_lda != 0;
        y.h = c.hartree != 0;
        y.pp = c.pseudo != 0;
        y.vloc = (const T*)e_vloc(e);
        y.tf_x = c.tf_x;
        y.vw_y = c.vw_y;
        y.dV = g->dV;
        y.invN = 1.0 / (double)g->N;
        y.ewald = c.ewald_energy;
        const size_t hb = (size_t)g->Nc * sizeof(C);
        y.RG = y.h ? (C*)b->sc.get("RG" + std::to_string(s), hb) : nullptr;
        y.SG = y.vw ? (C*)b->sc.get("SG" + std::to_string(s), hb) : nullptr;
        y.ktiles = (y.n2h + L - 1) / L;
        const long long nrows = (long long)y.n0 * y.n1;
        y.itA = (int)sysA.size();
        y.nA = (int)((nrows + R - 1) / R);
        for (int k = 0; k < y.nA; ++k) sysA.push_back(s);
        y.itB = (int)sysB.size();
        y.nB = y.n0 * y.ktiles;
        for (int k = 0; k < y.nB; ++k) sysB.push_back(s);
        y.itC = (int)sysC.size();
        y.nC = y.n1 * y.ktiles;
        for (int k = 0; k < y.nC; ++k) sysC.push_back(s);
    }
    b->nA = (int)sysA.size();
    b->nB = (int)sysB.size();
    b->nC = (int)sysC.size();
    b->h_sys.assign((unsigned char*)sys.data(), (unsigned char*)(sys.data() + S));
    cudaFree(b->d_sys);
    cudaFree(b->d_fft);
    cudaFree(b->d_tw);
    cudaFree(b->d_sysA);
    cudaFree(b->d_sysB);
    cudaFree(b->d_sysC);
    cudaFree(b->d_partA);
    cudaFree(b->d_partE);
    OFDFT_CK(cudaMalloc(&b->d_sys, S * sizeof(PbSys<T>)));
    OFDFT_CK(cudaMalloc(&b->d_fft, b->fft.size() * sizeof(PbFft)));
    OFDFT_CK(cudaMalloc(&b->d_tw, tw.size() * sizeof(C)));
    OFDFT_CK(cudaMalloc(&b->d_sysA, sysA.size() * sizeof(int)));
    OFDFT_CK(cudaMalloc(&b->d_sysB, sysB.size() * sizeof(int)));
    OFDFT_CK(cudaMalloc(&b->d_sysC, sysC.size() * sizeof(int)));
    OFDFT_CK(cudaMalloc(&b->d_partA, (size_t)b->nA * kPbSumsA * sizeof(double)));
    OFDFT_CK(cudaMalloc(&b->d_partE, (size_t)b->nA * kPbSumsE * sizeof(double)));
    upload_now(b->d_sys, sys.data(), S * sizeof(PbSys<T>));
    upload_now(b->d_fft, b->fft.data(), b->fft.size() * sizeof(PbFft));
    upload_now(b->d_tw, tw.data(), tw.size() * sizeof(C));
    upload_now(b->d_sysA, sysA.data(), sysA.size() * sizeof(int));
    upload_now(b->d_sysB, sysB.data(), sysB.size() * sizeof(int));
    upload_now(b->d_sysC, sysC.data(), sysC.size() * sizeof(int));
    // shared memory: two exchange buffers sized for the longest row tile and column tile
    int n2max = 0, nmax = 0;
    for (const PbSys<T>& y : sys) {
        n2max = std::max(n2max, y.n2);
        nmax = std::max(nmax, std::max(y.n0, y.n1));
    }
    const int slots = std::max(R * (n2max + 1), nmax * (L + 1));
    b->smem = 2 * (size_t)slots * sizeof(C);
    int per_sm = 0;
    OFDFT_CK(cudaFuncSetAttribute(k_pb_eval<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem));
    OFDFT_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pb_eval<T>, b->shape.block, b->smem));
    OFDFT_REQUIRE(per_sm > 0, "batched evaluation: launch shape does not fit an SM");
    int dev = 0, sms = 0;
    OFDFT_CK(cudaGetDevice(&dev));
    OFDFT_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    b->grid = std::min(per_sm * sms, std::max(std::max(b->nA, b->nB), std::max(b->nC, S)));
    b->bufslots = slots;
}

template <typename T>
void launch_t(ofdft_batch_eval* b, cudaStream_t st, void* d_sys) {
    PbArgs<T> a;
    a.sys = (PbSys<T>*)(d_sys ? d_sys : b->d_sys);
    a.S = b->S;
    a.act = b->d_act;
    a.fft = b->d_fft;
    a.tw = (const typename Cplx<T>::type*)b->d_tw;
    a.sysA = b->d_sysA;
    a.sysB = b->d_sysB;
    a.sysC = b->d_sysC;
    a.nA = b->nA;
    a.nB = b->nB;
    a.nC = b->nC;
    a.partA = b->d_partA;
    a.partE = b->d_partE;
    a.E = b->d_E;
    a.k = make_consts();
    a.rows = b->shape.rows;
    a.lines = b->shape.lines;
    a.bufslots = b->bufslots;
    void* args[] = {&a};
    OFDFT_CK(cudaLaunchCooperativeKernel((const void*)k_pb_eval<T>, dim3(b->grid), dim3(b->shape.block), args,
                                         b->smem, st));
}

void build(ofdft_batch_eval* b) {
    if (b->prec == OFDFT_F64) build_t<double>(b);
    else build_t<float>(b);
}

void launch(ofdft_batch_eval* b, cudaStream_t st, void* d_sys = nullptr) {
    if (b->prec == OFDFT_F64) launch_t<double>(b, st, d_sys);
    else launch_t<float>(b, st, d_sys);
}

// rho/V pointers of a call into the device descriptors (one small upload)
template <typename T>
void set_fields_t(ofdft_batch_eval* b, void* const* rho, void* const* v, cudaStream_t st) {
    PbSys<T>* h = (PbSys<T>*)b->h_sys.data();
    for (int s = 0; s < b->S; ++s) {
        h[s].rho = (const T*)rho[s];
        h[s].V = (T*)v[s];
    }
    OFDFT_CK(cudaMemcpyAsync(b->d_sys, h, b->S * sizeof(PbSys<T>), cudaMemcpyHostToDevice, st));
}

void set_fields(ofdft_batch_eval* b, void* const* rho, void* const* v, cudaStream_t st) {
    if (b->prec == OFDFT_F64) set_fields_t<double>(b, rho, v, st);
    else set_fields_t<float>(b, rho, v, st);
}

}  // namespace

// ------------------------------------------------ the batched optimiser's use
namespace {

template <typename T>
void* fieldset_sys_t(ofdft_batch_eval* b, void* const* rho, void* const* v) {
    std::vector<PbSys<T>> h(b->S);
    memcpy(h.data(), b->h_sys.data(), b->S * sizeof(PbSys<T>));
    for (int s = 0; s < b->S; ++s) {
        h[s].rho = (const T*)rho[s];
        h[s].V = (T*)v[s];
    }
    void* d = nullptr;
    OFDFT_CK(cudaMalloc(&d, b->S * sizeof(PbSys<T>)));
    upload_now(d, h.data(), b->S * sizeof(PbSys<T>));
    return d;
}

}  // namespace

// A batched evaluation for the optimiser, or nullptr when some system is not
// eligible.  rho/v: fields of every system the autotuner may use (v is
// overwritten).
ofdft_batch_eval* batch_eval_open(int n, ofdft_eval** evs, void* const* rho, void* const* v, cudaStream_t st) {
    for (int i = 0; i < n; ++i)
        if (!eligible(evs[i], nullptr) || e_grid(evs[i])->prec != e_grid(evs[0])->prec) return nullptr;
    ofdft_batch_eval* b = nullptr;
    const int rc = ofdft_batch_eval_create(n, evs, 1, rho, v, (ofdft_stream)st, &b);
    if (rc != OFDFT_OK) OFDFT_REQUIRE(false, "batched evaluation: %s", ofdft_last_error());
    OFDFT_CK(cudaStreamCreateWithFlags(&b->gst, cudaStreamNonBlocking));
    OFDFT_CK(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
    OFDFT_CK(cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming));
    return b;
}

void batch_eval_close(ofdft_batch_eval* b) { delete b; }

// Enqueue the evaluation of the systems with act[s] on st: rho[s] -> v[s].
// Energies are readable with batch_eval_energies once st has been synchronised.
void batch_eval_enqueue(ofdft_batch_eval* b, void* const* rho, void* const* v, const unsigned char* act,
                        cudaStream_t st) {
    std::vector<void*> key(rho, rho + b->S);
    key.insert(key.end(), v, v + b->S);
    ofdft_batch_eval::FieldSet* f = nullptr;
    for (auto& x : b->sets)
        if (x.key == key) f = &x;
    if (!f) {
        b->sets.emplace_back();
        f = &b->sets.back();
        f->key = key;
        f->d_sys = b->prec == OFDFT_F64 ? fieldset_sys_t<double>(b, rho, v) : fieldset_sys_t<float>(b, rho, v);
    }
    // the mask is read by the copy at its turn in the stream: fill it after the
    // previous evaluation's copies are done (the caller synchronised st since)
    for (int s = 0; s < b->S; ++s) b->h_act[s] = act[s] ? 1 : 0;
    OFDFT_CK(cudaEventRecord(b->fork_ev, st));
    OFDFT_CK(cudaStreamWaitEvent(b->gst, b->fork_ev, 0));
    if (!f->exec && !f->graph_failed) {
        cudaGraph_t graph = nullptr;
        bool ok = cudaStreamBeginCapture(b->gst, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            cudaMemcpyAsync(b->d_act, b->h_act, b->S, cudaMemcpyHostToDevice, b->gst);
            try {
                launch(b, b->gst, f->d_sys);
            } catch (const Error&) {
                ok = false;
            }
            cudaMemcpyAsync(b->h_E, b->d_E, (size_t)b->S * OFDFT_NE * sizeof(double), cudaMemcpyDeviceToHost,
                            b->gst);
            ok = cudaStreamEndCapture(b->gst, &graph) == cudaSuccess && ok && graph;
            if (ok) ok = cudaGraphInstantiate(&f->exec, graph, 0) == cudaSuccess;
            if (graph) cudaGraphDestroy(graph);
        }
        if (!ok) {
            // cooperative launches that cannot be captured here run uncaptured
            f->exec = nullptr;
            f->graph_failed = true;
            cudaGetLastError();
        }
    }
    if (f->exec) {
        OFDFT_CK(cudaGraphLaunch(f->exec, b->gst));
    } else {
        OFDFT_CK(cudaMemcpyAsync(b->d_act, b->h_act, b->S, cudaMemcpyHostToDevice, b->gst));
        launch(b, b->gst, f->d_sys);
        OFDFT_CK(cudaMemcpyAsync(b->h_E, b->d_E, (size_t)b->S * OFDFT_NE * sizeof(double), cudaMemcpyDeviceToHost,
                                 b->gst));
    }
    OFDFT_CK(cudaEventRecord(b->join_ev, b->gst));
    OFDFT_CK(cudaStreamWaitEvent(st, b->join_ev, 0));
}

// the total energy of system s of the last evaluation (after st was synchronised)
double batch_eval_energy(const ofdft_batch_eval* b, int s) { return b->h_E[(size_t)s * OFDFT_NE + OFDFT_E_TOTAL]; }
bool batch_eval_graphed(const ofdft_batch_eval* b) {
    for (const auto& f : b->sets)
        if (f.exec) return true;
    return false;
}

// ---------------------------------------------------------------- C ABI
extern "C" {

int ofdft_batch_eval_eligible(ofdft_eval* e) {
    if (!e) return 0;
    return eligible(e, nullptr) ? 1 : 0;
}

int ofdft_batch_eval_create(int n, ofdft_eval** evs, int tune, void* const* rho, void* const* v_work,
                            ofdft_stream s, ofdft_batch_eval** out) {
    return guard([&] {
        OFDFT_REQUIRE(out && evs && n > 0 && n <= kPbMaxSys, "ofdft_batch_eval_create: 1..%d evaluators", kPbMaxSys);
        *out = nullptr;
        auto* b = new ofdft_batch_eval();
        try {
            b->S = n;
            b->evs.assign(evs, evs + n);
            b->prec = e_grid(evs[0])->prec;
            std::string sig = b->prec == OFDFT_F64 ? "f64" : "f32";
            for (int i = 0; i < n; ++i) {
                OFDFT_REQUIRE(evs[i], "ofdft_batch_eval_create: null evaluator %d", i);
                std::string why;
                OFDFT_REQUIRE(eligible(evs[i], &why), "ofdft_batch_eval_create: system %d: %s", i, why.c_str());
                OFDFT_REQUIRE(e_grid(evs[i])->prec == b->prec, "ofdft_batch_eval_create: mixed precisions");
                const int* nr = e_grid(evs[i])->nr;
                sig += ":" + std::to_string(nr[0]) + "x" + std::to_string(nr[1]) + "x" + std::to_string(nr[2]);
            }
            b->sig = sig;
            OFDFT_CK(cudaMalloc(&b->d_E, (size_t)n * OFDFT_NE * sizeof(double)));
            OFDFT_CK(cudaMallocHost(&b->h_E, (size_t)n * OFDFT_NE * sizeof(double)));
            OFDFT_CK(cudaMalloc(&b->d_act, kPbMaxSys));
            OFDFT_CK(cudaMallocHost(&b->h_act, kPbMaxSys));
            memset(b->h_act, 1, kPbMaxSys);
            upload_now(b->d_act, b->h_act, kPbMaxSys);
            cudaStream_t st = (cudaStream_t)s;
            auto it = tuned_shapes().find(sig);
            if (it != tuned_shapes().end()) {
                b->shape = it->second;
                b->tuned_ms = it->second.ms;
                build(b);
            } else if (tune && rho && v_work) {
                // autotuner: every candidate shape that fits, timed on this batch
                const int blocks[] = {128, 256};
                const int rowss[] = {2, 4, 8};
                const int liness[] = {8, 16, 32};
                cudaEvent_t e0, e1;
                OFDFT_CK(cudaEventCreate(&e0));
                OFDFT_CK(cudaEventCreate(&e1));
                double best = 1e30;
                PbShape bs;
                for (int bk : blocks)
                    for (int r : rowss)
                        for (int l : liness) {
                            b->shape.block = bk;
                            b->shape.rows = r;
                            b->shape.lines = l;
                            try {
                                build(b);
                            } catch (const Error&) {
                                continue;  // shape does not fit
                            }
                            set_fields(b, rho, v_work, st);
                            launch(b, st);  // warm
                            OFDFT_CK(cudaEventRecord(e0, st));
                            for (int k = 0; k < 3; ++k) launch(b, st);
                            OFDFT_CK(cudaEventRecord(e1, st));
                            OFDFT_CK(cudaEventSynchronize(e1));
                            float ms = 0.f;
                            OFDFT_CK(cudaEventElapsedTime(&ms, e0, e1));
                            if (ms / 3.0 < best) {
                                best = ms / 3.0;
                                bs = b->shape;
                                bs.ms = best;
                            }
                        }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                OFDFT_REQUIRE(best < 1e30, "batched evaluation: no launch shape fits");
                b->shape = bs;
                b->tuned_ms = best;
                tuned_shapes()[sig] = bs;
                build(b);
            } else {
                build(b);
            }
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

int ofdft_batch_eval_run(ofdft_batch_eval* b, void* const* rho, void* const* v_out, const unsigned char* active,
                         double* energies, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(b && rho && v_out, "ofdft_batch_eval_run: null argument");
        cudaStream_t st = (cudaStream_t)s;
        for (int i = 0; i < b->S; ++i) {
            OFDFT_REQUIRE(rho[i] && v_out[i], "ofdft_batch_eval_run: null field of system %d", i);
            b->h_act[i] = active ? (active[i] ? 1 : 0) : 1;
        }
        OFDFT_CK(cudaMemcpyAsync(b->d_act, b->h_act, b->S, cudaMemcpyHostToDevice, st));
        set_fields(b, rho, v_out, st);
        launch(b, st);
        OFDFT_CK(cudaMemcpyAsync(b->h_E, b->d_E, (size_t)b->S * OFDFT_NE * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (energies) {
            OFDFT_CK(cudaStreamSynchronize(st));
            for (int i = 0; i < b->S; ++i)
                if (b->h_act[i])
                    for (int q = 0; q < OFDFT_NE; ++q) energies[(size_t)i * OFDFT_NE + q] = b->h_E[(size_t)i * OFDFT_NE + q];
        }
    });
}

int ofdft_batch_eval_shape(const ofdft_batch_eval* b, int* block, int* rows, int* lines, int* grid, double* tuned_ms) {
    return guard([&] {
        OFDFT_REQUIRE(b, "ofdft_batch_eval_shape: null handle");
        if (block) *block = b->shape.block;
        if (rows) *rows = b->shape.rows;
        if (lines) *lines = b->shape.lines;
        if (grid) *grid = b->grid;
        if (tuned_ms) *tuned_ms = b->tuned_ms;
    });
}

int ofdft_batch_eval_set_shape(ofdft_batch_eval* b, int block, int rows, int lines) {
    return guard([&] {
        OFDFT_REQUIRE(b, "ofdft_batch_eval_set_shape: null handle");
        OFDFT_REQUIRE((block == 128 || block == 256) && rows >= 1 && rows <= 16 && lines >= 1 && lines <= 64,
                      "ofdft_batch_eval_set_shape: block 128 or 256, rows 1..16, lines 1..64");
        b->shape.block = block;
        b->shape.rows = rows;
        b->shape.lines = lines;
        build(b);
        tuned_shapes()[b->sig] = b->shape;
    });
}

void ofdft_batch_eval_destroy(ofdft_batch_eval* b) { delete b; }

}  // extern "C"
