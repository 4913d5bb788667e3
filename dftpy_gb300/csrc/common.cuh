// Shared definitions of the GB300 OF-DFT library: error state, grid geometry,
// G vectors from indices, deterministic float64 block reductions, scratch.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/ofdft.h"

namespace ofdft {

// ----------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
const char* cufft_str(cufftResult r);

struct Error {
    int code;
};

#define OFDFT_CK(call)                                                                    \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            ::ofdft::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,                 \
                               cudaGetErrorString(e_));                                   \
            throw ::ofdft::Error{OFDFT_ECUDA};                                            \
        }                                                                                 \
    } while (0)

#define OFDFT_CF(call)                                                                    \
    do {                                                                                  \
        cufftResult r_ = (call);                                                          \
        if (r_ != CUFFT_SUCCESS) {                                                        \
            ::ofdft::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,                 \
                               ::ofdft::cufft_str(r_));                                   \
            throw ::ofdft::Error{OFDFT_ECUFFT};                                           \
        }                                                                                 \
    } while (0)

#define OFDFT_REQUIRE(cond, ...)                                                          \
    do {                                                                                  \
        if (!(cond)) {                                                                    \
            ::ofdft::set_error(__VA_ARGS__);                                              \
            throw ::ofdft::Error{OFDFT_EINVAL};                                           \
        }                                                                                 \
    } while (0)

#define OFDFT_LAUNCH_CHECK() OFDFT_CK(cudaGetLastError())

// Setup-time copies made without a caller stream (tables, ion lists).  A plain
// cudaMemcpy from pageable memory may return before its DMA lands and is not
// ordered before kernels on non-blocking streams, so these copies go through
// the calling thread's default stream and are waited for: when they return,
// kernels launched afterwards on any stream see the data.
inline void upload_now(void* dst, const void* src, size_t bytes) {
    OFDFT_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, cudaStreamPerThread));
    OFDFT_CK(cudaStreamSynchronize(cudaStreamPerThread));
}

inline void zero_now(void* dst, size_t bytes) {
    OFDFT_CK(cudaMemsetAsync(dst, 0, bytes, cudaStreamPerThread));
    OFDFT_CK(cudaStreamSynchronize(cudaStreamPerThread));
}

// Run a body and convert exceptions into the int status of the C ABI.
template <class F>
int guard(F&& f) {
    try {
        f();
        return OFDFT_OK;
    } catch (const Error& e) {
        return e.code;
    } catch (const std::bad_alloc&) {
        set_error("host out of memory");
        return OFDFT_ENOMEM;
    } catch (...) {
        set_error("unknown exception");
        return OFDFT_EINVAL;
    }
}

// ---------------------------------------------------------------- geometry
// Grid geometry passed by value to kernels.  G = f0*b0 + f1*b1 + f2*b2 with
// integer fftfreq/rfftfreq indices f times the factor numpy's fftfreq applies
// (1/(n*(1/n)), exactly 1 for the usual FFT sizes) and b the reciprocal rows.
struct Geo {
    int n0, n1, n2, n2h;
    long long N, Nc;
    double b[9];
    double fv[3];
    float bf[9];  // float copies for the FP32-mixed kernels
};

__host__ __device__ inline long long freq_index(int i, int n) {
    return (i < (n - 1) / 2 + 1) ? i : i - n;   // numpy fftfreq ordering
}

// G vector and |G|^2 of half-grid linear index idx, evaluated with the same
// operation order as the reference's einsum (no FMA contraction).
__device__ inline void gvec(const Geo& g, long long idx, double& gx, double& gy, double& gz, double& gg) {
    int k = (int)(idx % g.n2h);
    long long t = idx / g.n2h;
    int j = (int)(t % g.n1);
    int i = (int)(t / g.n1);
    double f0 = __dmul_rn((double)freq_index(i, g.n0), g.fv[0]);
    double f1 = __dmul_rn((double)freq_index(j, g.n1), g.fv[1]);
    double f2 = __dmul_rn((double)k, g.fv[2]);
    gx = __dadd_rn(__dadd_rn(__dmul_rn(f0, g.b[0]), __dmul_rn(f1, g.b[3])), __dmul_rn(f2, g.b[6]));
    gy = __dadd_rn(__dadd_rn(__dmul_rn(f0, g.b[1]), __dmul_rn(f1, g.b[4])), __dmul_rn(f2, g.b[7]));
    gz = __dadd_rn(__dadd_rn(__dmul_rn(f0, g.b[2]), __dmul_rn(f1, g.b[5])), __dmul_rn(f2, g.b[8]));
    gg = __dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(gz, gz));
}

__device__ inline double gsq(const Geo& g, long long idx) {
    double gx, gy, gz, gg;
    gvec(g, idx, gx, gy, gz, gg);
    return gg;
}

// |G|^2 in the working precision M: float64 as above, or float32 arithmetic
// for the FP32-mixed kernels (GB300 runs float64 at a small fraction of float32).
template <typename M>
__device__ inline M gsq_t(const Geo& g, long long idx);

template <>
__device__ inline double gsq_t<double>(const Geo& g, long long idx) {
    return gsq(g, idx);
}

// float32 |G|^2 of half-grid indices (i, j, k)
__device__ inline float gsq_f(const Geo& g, int i, int j, int k) {
    float f0 = (float)(i < (g.n0 - 1) / 2 + 1 ? i : i - g.n0);
    float f1 = (float)(j < (g.n1 - 1) / 2 + 1 ? j : j - g.n1);
    float f2 = (float)k;
    float gx = f0 * g.bf[0] + f1 * g.bf[3] + f2 * g.bf[6];
    float gy = f0 * g.bf[1] + f1 * g.bf[4] + f2 * g.bf[7];
    float gz = f0 * g.bf[2] + f1 * g.bf[5] + f2 * g.bf[8];
    return gx * gx + gy * gy + gz * gz;
}

template <>
__device__ inline float gsq_t<float>(const Geo& g, long long idx) {
    int k = (int)(idx % g.n2h);
    int t = (int)(idx / g.n2h);
    int j = t % g.n1;
    int i = t / g.n1;
    return gsq_f(g, i, j, k);
}

// Half-space mask that counts each +-G pair once (src/dftpy/grid.py:658-695,
// serial case), as a predicate on the half-grid index.
__device__ inline bool half_mask(const Geo& g, long long idx) {
    int k = (int)(idx % g.n2h);
    long long t = idx / g.n2h;
    int j = (int)(t % g.n1);
    int i = (int)(t / g.n1);
    int D0 = g.n0 / 2, D1 = g.n1 / 2, D2 = g.n2 / 2;
    int M0 = g.n0 % 2, M1 = g.n1 % 2, M2 = g.n2 % 2;
    if (k == 0) {
        if (i == 0 && j > D1) return false;
        if (i > D0) return false;
        if (M0 == 0 && i == D0 && j > D1) return false;
        if (M0 == 0 && M1 == 0 && i == D0 && j == D1) return false;
        if (M1 == 0 && i == 0 && j == D1) return false;
    }
    if (M2 == 0 && k == D2) {
        if (i == 0 && j == 0) return false;
        if (i == 0 && j > D1) return false;
        if (i > D0) return false;
        if (M1 == 0 && i == 0 && j == D1) return false;
        if (M0 == 0 && i == D0 && j == 0) return false;
        if (M0 == 0 && i == D0 && j > D1) return false;
    }
    if (M0 == 0 && M1 == 0 && M2 == 0 && i == D0 && j == D1 && k == D2) return false;
    return true;
}

// ------------------------------------------------------------- reductions
// Each block reduces NS float64 sums with a fixed tree and writes them to
// partials[blockIdx.x * NS + s]; reduce_finalize sums the block partials in a
// fixed order.  Launch shapes are fixed per grid, so results are bit-stable.
constexpr int RED_THREADS = 256;

template <int NS>
__device__ inline void block_sum_store(double (&v)[NS], double* partials) {
    __shared__ double sh[NS][RED_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        double x = v[s];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[s][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x / 32;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            double x = (lane < nw) ? sh[s][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) partials[(long long)blockIdx.x * NS + s] = x;
        }
    }
}

// The same block sum, stored at partials[slot * NS + s] (a block of a batched
// launch stores at its position in the launch).
template <int NS>
__device__ inline void block_sum_store_at(double (&v)[NS], double* partials, long long slot) {
    __shared__ double sh[NS][RED_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        double x = v[s];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[s][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x / 32;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            double x = (lane < nw) ? sh[s][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) partials[slot * NS + s] = x;
        }
    }
}

// min/max helpers: kind 0 = sum, 1 = min, 2 = max
__device__ inline double red_op(double a, double b, int kind) {
    return kind == 0 ? a + b : (kind == 1 ? fmin(a, b) : fmax(a, b));
}

template <int NS>
__device__ inline void block_reduce_store(double (&v)[NS], const int (&kind)[NS], double* partials) {
    __shared__ double sh[NS][RED_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        double x = v[s];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = red_op(x, __shfl_down_sync(0xffffffffu, x, o), kind[s]);
        if (lane == 0) sh[s][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x / 32;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            double id = kind[s] == 0 ? 0.0 : (kind[s] == 1 ? INFINITY : -INFINITY);
            double x = (lane < nw) ? sh[s][lane] : id;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x = red_op(x, __shfl_down_sync(0xffffffffu, x, o), kind[s]);
            if (lane == 0) partials[(long long)blockIdx.x * NS + s] = x;
        }
    }
}

// reduce nblk x ns partials into out[ns]; kinds: bit pattern 2 bits per slot
__global__ void reduce_finalize(const double* partials, int nblk, int ns, unsigned long long kinds, double* out);

// ------------------------------------------------------------------ scratch
// Named device buffers that grow on demand and live as long as their owner.
class Scratch {
public:
    ~Scratch();
    void* get(const std::string& name, size_t bytes);
    void release_all();
    size_t total() const;

private:
    struct Buf {
        void* p = nullptr;
        size_t n = 0;
    };
    std::map<std::string, Buf> bufs_;
};

template <typename T>
struct Cplx;
template <>
struct Cplx<double> {
    using type = cufftDoubleComplex;
};
template <>
struct Cplx<float> {
    using type = cufftComplex;
};

// default 1-D launch shape for grid-stride kernels
inline int blocks_for(long long n, int threads, int max_blocks) {
    long long b = (n + threads - 1) / threads;
    if (b > max_blocks) b = max_blocks;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace ofdft

// ------------------------------------------------------------------- grid
struct ofdft_grid {
    int nr[3];
    int n2h;
    long long N, Nc;
    double lattice[9];
    double rlattice[9];  // rows b_j = 2 pi inv(lattice)^T rows
    double volume, dV;
    int prec;
    size_t esize;
    ofdft::Geo geo;
    int sms;
    int red_blocks;                       // fixed block count of field reductions
    std::map<long long, cufftHandle> plans;  // key = dir*1e6 + batch
    ofdft::Scratch scratch;
    double* d_partials = nullptr;         // red_blocks * 32 doubles
    double* d_results = nullptr;          // 64 doubles
    double* h_results = nullptr;          // pinned mirror

    cufftHandle plan(int dir, int batch);  // dir 0: R2C, 1: C2R
    void exec_r2c(const void* in, void* out, int batch, cudaStream_t s);
    void exec_c2r(void* in, void* out, int batch, cudaStream_t s);
    size_t real_bytes() const { return (size_t)N * esize; }
    size_t cplx_bytes() const { return (size_t)Nc * 2 * esize; }
};
