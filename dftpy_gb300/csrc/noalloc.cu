// A float64 field reduction that allocates nothing.
//
// Some callers of this library cannot allocate device memory at the point
// where they need a reduction: code running inside an allocator callback or a
// memory-pool hook (a cudaMalloc there would re-enter the allocator), hosts
// that forbid allocation after start-up (real-time or safety-certified
// loops), or a process whose device memory is fully reserved by a framework
// pool.  ofdft_dot uses a grid handle whose scratch was allocated when the
// handle was created; ofdft_dot_noalloc needs no handle and no allocation.
//
// Its scratch is the file-scope array g_noalloc_partials below: 4096 float64
// block partials (32 KiB).  The array lives in the module image, so every GPU
// that loads this library holds those 32 KiB until the process exits.
//
// Limits and behaviour:
//   * n must be in 1 .. kNoAllocMaxElems (4096 blocks x 16384 elements =
//     67,108,864, e.g. a 406^3 grid); larger n is rejected with OFDFT_EINVAL.
//   * The first call on each device looks the array's device address up with
//     cudaGetSymbolAddress (with that device current), caches it, and queries
//     the attributes of all three kernels.  Under CUDA's lazy module loading
//     those steps make the driver load this module's code and the array onto
//     the device, which takes device memory; after them no later call loads
//     anything.  So make the first call on each device at start-up, before a
//     pool reserves the device's memory and before any stream capture.
//   * All calls share the one array and it keeps the last call's contents.
//     Every partial a call reads is written earlier in the same call, so no
//     clearing is needed, but two calls that overlap on the GPU (different
//     streams, no ordering between them) race on the array.
#include "common.cuh"

#include <mutex>

namespace {

constexpr int kNoAllocBlocks = 4096;
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 64;
constexpr long long kNoAllocChunk = (long long)kNoAllocThreads * kNoAllocPerThread;  // elements per block
constexpr long long kNoAllocMaxElems = (long long)kNoAllocBlocks * kNoAllocChunk;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocBlocks];

// Each block sums one contiguous chunk of a*b (or a) in float64 and writes its
// partial; the block count is ceil(n / chunk), so results are bit-stable.
template <typename T>
__global__ void __launch_bounds__(kNoAllocThreads) k_noalloc_partial(const T* __restrict__ a,
                                                                     const T* __restrict__ b, long long n,
                                                                     double* partials) {
    const long long base = (long long)blockIdx.x * kNoAllocChunk;
    double acc = 0.0;
    for (int k = 0; k < kNoAllocPerThread; ++k) {
        const long long i = base + (long long)k * kNoAllocThreads + threadIdx.x;
        if (i < n) acc += b ? (double)a[i] * (double)b[i] : (double)a[i];
    }
    __shared__ double sh[kNoAllocThreads / 32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double x = threadIdx.x < kNoAllocThreads / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (threadIdx.x == 0) partials[blockIdx.x] = x;
    }
}

// One block sums the nblk partials in a fixed order into *out (device memory).
__global__ void __launch_bounds__(kNoAllocThreads) k_noalloc_final(const double* partials, int nblk, double* out) {
    __shared__ double sh[kNoAllocThreads];
    double x = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kNoAllocThreads) x += partials[b];
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_partials on the current device, looked up once.
double* noalloc_scratch() {
    int dev = -1;
    OFDFT_CK(cudaGetDevice(&dev));
    OFDFT_REQUIRE(dev >= 0 && dev < kMaxDevices, "ofdft_dot_noalloc: device %d outside 0..%d", dev,
                  kMaxDevices - 1);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        OFDFT_CK(cudaGetSymbolAddress(&p, g_noalloc_partials));
        // load every kernel of this entry point now, so that no later call (a
        // float32 call after float64 ones, say) makes the driver load code
        cudaFuncAttributes fa;
        OFDFT_CK(cudaFuncGetAttributes(&fa, k_noalloc_partial<double>));
        OFDFT_CK(cudaFuncGetAttributes(&fa, k_noalloc_partial<float>));
        OFDFT_CK(cudaFuncGetAttributes(&fa, k_noalloc_final));
        g_noalloc_ptr[dev] = (double*)p;
    }
    return g_noalloc_ptr[dev];
}

}  // namespace

extern "C" int ofdft_dot_noalloc(const void* a, const void* b, long long n, int precision, double* out_dev,
                                 ofdft_stream s) {
    return ofdft::guard([&] {
        OFDFT_REQUIRE(a && out_dev, "ofdft_dot_noalloc: null argument");
        OFDFT_REQUIRE(precision == OFDFT_F64 || precision == OFDFT_F32, "ofdft_dot_noalloc: bad precision");
        OFDFT_REQUIRE(n >= 1 && n <= kNoAllocMaxElems,
                      "ofdft_dot_noalloc: n = %lld outside 1..%lld (the static scratch holds %d block partials "
                      "of %lld elements)",
                      n, kNoAllocMaxElems, kNoAllocBlocks, kNoAllocChunk);
        double* partials = noalloc_scratch();
        const int nblk = (int)((n + kNoAllocChunk - 1) / kNoAllocChunk);
        cudaStream_t st = (cudaStream_t)s;
        if (precision == OFDFT_F64)
            k_noalloc_partial<double><<<nblk, kNoAllocThreads, 0, st>>>((const double*)a, (const double*)b, n,
                                                                       partials);
        else
            k_noalloc_partial<float><<<nblk, kNoAllocThreads, 0, st>>>((const float*)a, (const float*)b, n,
                                                                      partials);
        OFDFT_LAUNCH_CHECK();
        k_noalloc_final<<<1, kNoAllocThreads, 0, st>>>(partials, nblk, out_dev);
        OFDFT_LAUNCH_CHECK();
    });
}
