// Float32 tile FFTs for the fused density-dependent-kernel pipeline.
//
// A line of N complex points is held by T = N/E threads with E points each:
// thread t holds element t + T*e in register e.  The transform is a Stockham
// auto-sort FFT (decimation in time): passes of radix E (one butterfly per
// thread) followed by at most one smaller radix (E/R butterflies per thread),
// exchanging through shared memory between passes.  On return register e holds
// output element t + T*e, the distribution of the input, so a line is loaded
// from and stored to the same addresses.  Twiddles come from a table of
// exp(-2 pi i k/N) computed on the host in float64; inverse transforms use its
// conjugate.  Transforms are unnormalised, as cuFFT's are.
//
// Real transforms along the contiguous axis use the half-length complex
// transform: z[m] = x[2m] + i x[2m+1] with the usual pre/post-processing of
// the pairs (k, H-k), H = n/2.  The C2R drops the imaginary parts of X[0] and
// X[H], as numpy's irfftn does.
#pragma once
#include "common.cuh"

#include <type_traits>

namespace ofdft {
namespace fz {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// a * (S i) with S = -1 (forward) or +1 (inverse)
template <int S>
__device__ __forceinline__ float2 mul_si(float2 a) {
    return S < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}
// a * (c + S s i)
template <int S>
__device__ __forceinline__ float2 mul_cs(float2 a, float c, float s) {
    const float ss = S < 0 ? -s : s;
    return make_float2(a.x * c - a.y * ss, a.x * ss + a.y * c);
}

constexpr float kC1 = 0.923879532511286756f;  // cos(pi/8)
constexpr float kS1 = 0.382683432365089772f;  // sin(pi/8)
constexpr float kH = 0.707106781186547524f;   // cos(pi/4)

// In-register DFTs, natural order in and out; X[k] = sum_n x[n] exp(S 2 pi i nk/R)
template <int S>
__device__ __forceinline__ void dft2(float2* v) {
    const float2 a = v[0];
    v[0] = cadd(a, v[1]);
    v[1] = csub(a, v[1]);
}

template <int S>
__device__ __forceinline__ void dft4(float2* v) {
    const float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    const float2 a2 = cadd(v[1], v[3]), a3 = mul_si<S>(csub(v[1], v[3]));
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, a3);
    v[3] = csub(a1, a3);
}

// 8 and 16 points: radix-2 split, X[k] = E[k] + W^k O[k], X[k + R/2] = E[k] - W^k O[k]
template <int S>
__device__ __forceinline__ void dft8(float2* v) {
    float2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft4<S>(e);
    dft4<S>(o);
    const float2 w1 = mul_cs<S>(o[1], kH, kH), w2 = mul_si<S>(o[2]), w3 = mul_cs<S>(o[3], -kH, kH);
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], w1);
    v[5] = csub(e[1], w1);
    v[2] = cadd(e[2], w2);
    v[6] = csub(e[2], w2);
    v[3] = cadd(e[3], w3);
    v[7] = csub(e[3], w3);
}

template <int S>
__device__ __forceinline__ void dft16(float2* v) {
    float2 e[8], o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        e[k] = v[2 * k];
        o[k] = v[2 * k + 1];
    }
    dft8<S>(e);
    dft8<S>(o);
    float2 w[8];
    w[0] = o[0];
    w[1] = mul_cs<S>(o[1], kC1, kS1);
    w[2] = mul_cs<S>(o[2], kH, kH);
    w[3] = mul_cs<S>(o[3], kS1, kC1);
    w[4] = mul_si<S>(o[4]);
    w[5] = mul_cs<S>(o[5], -kS1, kC1);
    w[6] = mul_cs<S>(o[6], -kH, kH);
    w[7] = mul_cs<S>(o[7], -kC1, kS1);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = cadd(e[k], w[k]);
        v[k + 8] = csub(e[k], w[k]);
    }
}

template <int R, int S>
__device__ __forceinline__ void dft(float2* v) {
    if constexpr (R == 2) dft2<S>(v);
    else if constexpr (R == 4) dft4<S>(v);
    else if constexpr (R == 8) dft8<S>(v);
    else {
        static_assert(R == 16, "radix must be 2, 4, 8 or 16");
        dft16<S>(v);
    }
}

// Shared-memory placement of element n of a line.
// Column tiles: 16 lines side by side, element-major, one pad slot per 16 elements.
struct ColIdx {
    __device__ __forceinline__ int operator()(int n) const { return n * 16 + (n >> 4); }
};
// Row tiles: one line per row buffer, one pad slot per 8 elements.
struct RowIdx {
    __device__ __forceinline__ int operator()(int n) const { return n + (n >> 3); }
};
// slots a line of n elements occupies
__host__ __device__ constexpr int col_slots(int n) { return n * 16 + (n >> 4) + 16; }
__host__ __device__ constexpr int row_slots(int n) { return n + (n >> 3) + 1; }

// radix of the pass that starts at sub-transform length NS
template <int N, int E, int NS>
struct PassRadix {
    static constexpr int R = (N / NS >= E) ? E : N / NS;
};

// One Stockham pass and, recursively, the passes after it.  sm must be free
// (every thread done with it) on entry; on return the last pass has read sm.
template <int N, int E, int S, int NS, class Idx>
struct Stockham {
    static constexpr int T = N / E;
    static constexpr int R = PassRadix<N, E, NS>::R;
    static constexpr int NB = E / R;
    static constexpr bool LAST = NS * R == N;
    static_assert(E % R == 0, "radix must divide the points per thread");

    __device__ __forceinline__ static void run(float2 (&v)[E], float2* sm, Idx ix, int t,
                                               const float2* __restrict__ tw) {
        __builtin_assume(t >= 0 && t < T);
        if constexpr (NS > 1) {
            __syncthreads();  // the previous pass's outputs are in sm
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = sm[ix(t + T * e)];
            if constexpr (!LAST) __syncthreads();  // every input read before sm is overwritten
        }
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            const int j = t + T * b;
            const int jm = j & (NS - 1);
            float2 u[R];
#pragma unroll
            for (int r = 0; r < R; ++r) u[r] = v[b + r * NB];
            if constexpr (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    const float2 w = __ldg(tw + r * jm * (N / (NS * R)));
                    u[r] = S < 0 ? cmul(u[r], w) : cmulc(u[r], w);
                }
            }
            dft<R, S>(u);
            if constexpr (LAST) {
#pragma unroll
                for (int r = 0; r < R; ++r) v[b + r * NB] = u[r];
            } else {
                const int idxD = (j / NS) * NS * R + jm;
#pragma unroll
                for (int r = 0; r < R; ++r) sm[ix(idxD + r * NS)] = u[r];
            }
        }
        if constexpr (!LAST) Stockham<N, E, S, NS * R, Idx>::run(v, sm, ix, t, tw);
    }
};

template <int N, int E, int S, class Idx>
__device__ __forceinline__ void line_fft(float2 (&v)[E], float2* sm, Idx ix, int t, const float2* __restrict__ tw) {
    Stockham<N, E, S, 1, Idx>::run(v, sm, ix, t, tw);
}

// Row placement: one pad slot per 16 elements.  With 8 points per thread the
// loads of every pass (16 consecutive elements per half-warp) and the stores
// of the first radix-8 pass fall in distinct banks; the second radix-8 pass of
// a 128-point row stores with a two-way conflict.  The offsets fold to
// immediates (thread t < 16 holds elements t + 16e), where an XOR swizzle
// free of conflicts costs integer instructions on every access.
struct RowPad16 {
    __device__ __forceinline__ int operator()(int n) const { return n + (n >> 4); }
};
// Second exchange buffer of the ping-pong row transforms: 8 pad slots per 64
// elements.  The second radix-8 pass stores elements n and n + 64 from
// threads t and t + 8; this places them 8 banks apart, so that store and the
// following loads are free of conflicts for 128- and 256-point rows.
struct RowPad8of64 {
    __device__ __forceinline__ int operator()(int n) const { return n + 8 * (n >> 6); }
};
template <int N>
struct RowLayout {
    using Idx = RowPad16;       // exchange buffer 0
    using Idx1 = RowPad8of64;   // exchange buffer 1
    static constexpr int slots = N + (N >> 4) + 1;
    static constexpr int slots1 = N + 8 * (N >> 6) + 1;
};

// The Stockham passes with two exchange buffers used in turn: pass p stores
// into buffer p & 1 and pass p + 1 reads it after one barrier, so a pass needs
// one barrier instead of two.  Entry: buffer 0 is free.  Exit: both buffers are
// free for the next transform (a trailing barrier is added when the number of
// exchanges is odd, because the last reads then come from buffer 0).
template <int N, int E, int S, int NS, int PASS, class Idx>
struct StockhamPP {
    static constexpr int T = N / E;
    static constexpr int R = PassRadix<N, E, NS>::R;
    static constexpr int NB = E / R;
    static constexpr bool LAST = NS * R == N;
    static_assert(E % R == 0, "radix must divide the points per thread");

    __device__ __forceinline__ static void run(float2 (&v)[E], float2* b0, float2* b1, Idx ix, int t,
                                               const float2* __restrict__ tw) {
        __builtin_assume(t >= 0 && t < T);
        if constexpr (NS > 1) {
            const float2* src = ((PASS - 1) & 1) ? b1 : b0;
            __syncthreads();  // the previous pass's outputs are in src
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = src[ix(t + T * e)];
        }
        float2* dst = (PASS & 1) ? b1 : b0;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            const int j = t + T * b;
            const int jm = j & (NS - 1);
            float2 u[R];
#pragma unroll
            for (int r = 0; r < R; ++r) u[r] = v[b + r * NB];
            if constexpr (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    const float2 w = __ldg(tw + r * jm * (N / (NS * R)));
                    u[r] = S < 0 ? cmul(u[r], w) : cmulc(u[r], w);
                }
            }
            dft<R, S>(u);
            if constexpr (LAST) {
#pragma unroll
                for (int r = 0; r < R; ++r) v[b + r * NB] = u[r];
            } else {
                const int idxD = (j / NS) * NS * R + jm;
#pragma unroll
                for (int r = 0; r < R; ++r) dst[ix(idxD + r * NS)] = u[r];
            }
        }
        if constexpr (!LAST) {
            StockhamPP<N, E, S, NS * R, PASS + 1, Idx>::run(v, b0, b1, ix, t, tw);
        } else if constexpr ((PASS & 1) == 1) {
            __syncthreads();  // odd number of exchanges: the last reads were from buffer 0
        }
    }
};

// ---- twiddles held in registers
// Every pass after the first multiplies by twiddles that depend only on the
// thread index, so a thread can load them once and keep them for all the
// lines it transforms.  tw_count<N, E>() is the number of such twiddles per
// thread; pass p's twiddle (b, r) sits at its offset + b * (R - 1) + r - 1.
template <int N, int E>
__host__ __device__ constexpr int tw_count() {
    int c = 0;
    for (int ns = 1; ns < N;) {
        const int r = (N / ns >= E) ? E : N / ns;
        if (ns > 1) c += (E / r) * (r - 1);
        ns *= r;
    }
    return c;
}

template <int N, int E, int NS, int OFF>
struct TwFill {
    static constexpr int T = N / E;
    static constexpr int R = PassRadix<N, E, NS>::R;
    static constexpr int NB = E / R;
    static constexpr bool LAST = NS * R == N;
    __device__ __forceinline__ static void run(float2* w, int t, const float2* __restrict__ tw) {
        constexpr int HERE = NS > 1 ? NB * (R - 1) : 0;
        if constexpr (NS > 1) {
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                const int jm = (t + T * b) & (NS - 1);
#pragma unroll
                for (int r = 1; r < R; ++r) w[OFF + b * (R - 1) + r - 1] = __ldg(tw + r * jm * (N / (NS * R)));
            }
        }
        if constexpr (!LAST) TwFill<N, E, NS * R, OFF + HERE>::run(w, t, tw);
    }
};

// loads this thread's twiddles of an N-point line transform (t < N / E)
template <int N, int E>
__device__ __forceinline__ void tw_load(float2 (&w)[tw_count<N, E>()], int t, const float2* __restrict__ tw) {
    TwFill<N, E, 1, 0>::run(w, t, tw);
}

// The Stockham passes with register twiddles (OFF: this pass's first twiddle)
// and one exchange buffer (PP false: two barriers per exchange) or two used in
// turn (PP true: one barrier per exchange, as StockhamPP).
template <int N, int E, int S, int NS, int PASS, int OFF, bool PP, class Idx, class Idx1 = Idx>
struct StockhamR {
    static constexpr int T = N / E;
    static constexpr int R = PassRadix<N, E, NS>::R;
    static constexpr int NB = E / R;
    static constexpr bool LAST = NS * R == N;
    static_assert(E % R == 0, "radix must divide the points per thread");

    // element n of buffer 1 sits at ix1(n) (PP only; buffer 0 uses ix)
    template <int B>
    __device__ __forceinline__ static int at(Idx ix, Idx1 ix1, int n) {
        if constexpr (B == 1) return ix1(n);
        else return ix(n);
    }

    __device__ __forceinline__ static void run(float2 (&v)[E], float2* b0, float2* b1, Idx ix, int t,
                                               const float2* w, Idx1 ix1 = Idx1()) {
        __builtin_assume(t >= 0 && t < T);
        constexpr int HERE = NS > 1 ? NB * (R - 1) : 0;
        constexpr int SB = PP ? ((PASS - 1) & 1) : 0;  // buffer this pass reads
        constexpr int DB = PP ? (PASS & 1) : 0;        // buffer this pass writes
        const float2* src = SB ? b1 : b0;
        float2* dst = DB ? b1 : b0;
        if constexpr (NS > 1) {
            __syncthreads();  // the previous pass's outputs are in src
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = src[at<SB>(ix, ix1, t + T * e)];
            if constexpr (!PP && !LAST) __syncthreads();  // every input read before the buffer is overwritten
        }
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            const int j = t + T * b;
            const int jm = j & (NS - 1);
            float2 u[R];
#pragma unroll
            for (int r = 0; r < R; ++r) u[r] = v[b + r * NB];
            if constexpr (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    const float2 tw = w[OFF + b * (R - 1) + r - 1];
                    u[r] = S < 0 ? cmul(u[r], tw) : cmulc(u[r], tw);
                }
            }
            dft<R, S>(u);
            if constexpr (LAST) {
#pragma unroll
                for (int r = 0; r < R; ++r) v[b + r * NB] = u[r];
            } else {
                const int idxD = (j / NS) * NS * R + jm;
#pragma unroll
                for (int r = 0; r < R; ++r) dst[at<DB>(ix, ix1, idxD + r * NS)] = u[r];
            }
        }
        if constexpr (!LAST) {
            StockhamR<N, E, S, NS * R, PASS + 1, OFF + HERE, PP, Idx, Idx1>::run(v, b0, b1, ix, t, w, ix1);
        } else if constexpr (PP && (PASS & 1) == 1) {
            __syncthreads();  // odd number of exchanges: the last reads were from buffer 0
        }
    }
};

// single exchange buffer `sm`, free on entry; the last pass has read it on return
template <int N, int E, int S, class Idx>
__device__ __forceinline__ void line_fft_r(float2 (&v)[E], float2* sm, Idx ix, int t, const float2* w) {
    StockhamR<N, E, S, 1, 0, 0, false, Idx>::run(v, sm, sm, ix, t, w);
}
// two exchange buffers used in turn (entry: b0 free; exit: both free), laid out
// by ix and ix1
template <int N, int E, int S, class Idx, class Idx1>
__device__ __forceinline__ void line_fft_ppr(float2 (&v)[E], float2* b0, float2* b1, Idx ix, Idx1 ix1, int t,
                                             const float2* w) {
    StockhamR<N, E, S, 1, 0, 0, true, Idx, Idx1>::run(v, b0, b1, ix, t, w, ix1);
}

// ---- 1-D bulk asynchronous copies (TMA) into shared memory, completed on an
// mbarrier.  Sources and destinations are 16-byte aligned, sizes multiples of 16.
__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// makes initialised mbarriers visible to the copy engine
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// orders this thread's earlier shared-memory accesses before later copies into it
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// Elapsed-time limit of an mbarrier wait: a bulk copy of a few tens of KB
// completes in microseconds, so 100 ms means the copy is not coming.
constexpr unsigned long long kMbarWaitNs = 100000000ull;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool mbar_try(unsigned a, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    return done != 0;
}
// Waits for the phase of `parity` to complete for at most kMbarWaitNs of
// elapsed time (%globaltimer, read only once the first try has failed);
// false when it did not complete (the caller records an error instead of
// hanging).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    const unsigned a = smem_addr(bar);
    if (mbar_try(a, parity)) return true;
    const unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (mbar_try(a, parity)) return true;
        if (globaltimer_ns() - t0 > kMbarWaitNs) return false;
    }
}

template <int N, int E, int S, class Idx>
__device__ __forceinline__ void line_fft_pp(float2 (&v)[E], float2* b0, float2* b1, Idx ix, int t,
                                            const float2* __restrict__ tw) {
    StockhamPP<N, E, S, 1, 0, Idx>::run(v, b0, b1, ix, t, tw);
}

}  // namespace fz
}  // namespace ofdft
