// Grid handle, cuFFT plans, DirectField.fft / ReciprocalField.ifft and
// float64 field reductions of the C ABI.
#include "common.cuh"

#include <algorithm>

#include <cstring>
#include <mutex>

namespace ofdft {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

const char* cufft_str(cufftResult r) {
    switch (r) {
        case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
        case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
        case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
        case CUFFT_INVALID_TYPE: return "CUFFT_INVALID_TYPE";
        case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
        case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
        case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
        case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
        case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
        default: return "cuFFT error";
    }
}

__global__ void reduce_finalize(const double* partials, int nblk, int ns, unsigned long long kinds, double* out) {
    __shared__ double sh[RED_THREADS];
    for (int s = 0; s < ns; ++s) {
        int kind = (int)((kinds >> (2 * s)) & 3ull);
        double id = kind == 0 ? 0.0 : (kind == 1 ? INFINITY : -INFINITY);
        double x = id;
        for (int b = threadIdx.x; b < nblk; b += blockDim.x) x = red_op(x, partials[(long long)b * ns + s], kind);
        sh[threadIdx.x] = x;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) sh[threadIdx.x] = red_op(sh[threadIdx.x], sh[threadIdx.x + w], kind);
            __syncthreads();
        }
        if (threadIdx.x == 0) out[s] = sh[0];
        __syncthreads();
    }
}

Scratch::~Scratch() { release_all(); }

void* Scratch::get(const std::string& name, size_t bytes) {
    Buf& b = bufs_[name];
    if (b.n < bytes) {
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.n = 0;
        cudaError_t e = cudaMalloc(&b.p, bytes);
        if (e != cudaSuccess) {
            b.p = nullptr;
            cudaGetLastError();
            set_error("cudaMalloc of %zu bytes for '%s' failed: %s", bytes, name.c_str(), cudaGetErrorString(e));
            throw Error{OFDFT_ENOMEM};
        }
        b.n = bytes;
    }
    return b.p;
}

void Scratch::release_all() {
    for (auto& kv : bufs_)
        if (kv.second.p) cudaFree(kv.second.p);
    bufs_.clear();
}

size_t Scratch::total() const {
    size_t t = 0;
    for (auto& kv : bufs_) t += kv.second.n;
    return t;
}

// ------------------------------------------------------------ field kernels
template <typename T>
__global__ void k_scale_copy(const T* __restrict__ a, T* __restrict__ b, long long n, double s) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (T)((double)a[i] * s);
}

template <typename T>
__global__ void k_dot(const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ c, long long n,
                      double* partials) {
    double v[1] = {0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double x = (double)a[i];
        if (b) x *= (double)b[i];
        if (c) x *= (double)c[i];
        v[0] += x;
    }
    block_sum_store<1>(v, partials);
}

}  // namespace ofdft

using namespace ofdft;

cufftHandle ofdft_grid::plan(int dir, int batch) {
    long long key = (long long)dir * 1000000LL + batch;
    auto it = plans.find(key);
    if (it != plans.end()) return it->second;
    cufftHandle h;
    OFDFT_CF(cufftCreate(&h));
    int n[3] = {nr[0], nr[1], nr[2]};
    cufftType t;
    if (prec == OFDFT_F64) t = dir == 0 ? CUFFT_D2Z : CUFFT_Z2D;
    else t = dir == 0 ? CUFFT_R2C : CUFFT_C2R;
    int idist = dir == 0 ? (int)N : (int)Nc;
    int odist = dir == 0 ? (int)Nc : (int)N;
    size_t ws = 0;
    cufftResult r = cufftMakePlanMany(h, 3, n, nullptr, 1, idist, nullptr, 1, odist, t, batch, &ws);
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(h);
        set_error("cufftMakePlanMany(%d,%d,%d, batch %d) failed: %s", nr[0], nr[1], nr[2], batch, cufft_str(r));
        throw Error{OFDFT_ECUFFT};
    }
    plans[key] = h;
    return h;
}

void ofdft_grid::exec_r2c(const void* in, void* out, int batch, cudaStream_t s) {
    cufftHandle h = plan(0, batch);
    OFDFT_CF(cufftSetStream(h, s));
    if (prec == OFDFT_F64) OFDFT_CF(cufftExecD2Z(h, (cufftDoubleReal*)in, (cufftDoubleComplex*)out));
    else OFDFT_CF(cufftExecR2C(h, (cufftReal*)in, (cufftComplex*)out));
}

void ofdft_grid::exec_c2r(void* in, void* out, int batch, cudaStream_t s) {
    cufftHandle h = plan(1, batch);
    OFDFT_CF(cufftSetStream(h, s));
    if (prec == OFDFT_F64) OFDFT_CF(cufftExecZ2D(h, (cufftDoubleComplex*)in, (cufftDoubleReal*)out));
    else OFDFT_CF(cufftExecC2R(h, (cufftComplex*)in, (cufftReal*)out));
}

extern "C" {

const char* ofdft_last_error(void) { return ofdft::g_last_error.c_str(); }
const char* ofdft_version(void) { return "dftpy_gb300 ofdft 0.1 (sm_103a)"; }

int ofdft_grid_create(const int nr[3], const double lattice[9], int precision, ofdft_grid** out) {
    return guard([&] {
        OFDFT_REQUIRE(nr && lattice && out, "ofdft_grid_create: null argument");
        OFDFT_REQUIRE(nr[0] > 1 && nr[1] > 1 && nr[2] > 1, "ofdft_grid_create: grid must be > 1 per axis");
        OFDFT_REQUIRE(precision == OFDFT_F64 || precision == OFDFT_F32, "ofdft_grid_create: bad precision");
        long long N = (long long)nr[0] * nr[1] * nr[2];
        OFDFT_REQUIRE(N < (1LL << 31), "ofdft_grid_create: grid too large for 32-bit cuFFT strides");
        auto* g = new ofdft_grid();
        for (int d = 0; d < 3; ++d) g->nr[d] = nr[d];
        memcpy(g->lattice, lattice, 9 * sizeof(double));
        g->n2h = nr[2] / 2 + 1;
        g->N = N;
        g->Nc = (long long)nr[0] * nr[1] * g->n2h;
        const double* a = lattice;
        double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                     a[2] * (a[3] * a[7] - a[4] * a[6]);
        OFDFT_REQUIRE(det != 0.0, "ofdft_grid_create: singular lattice");
        double inv[9];  // inverse of the row matrix a
        inv[0] = (a[4] * a[8] - a[5] * a[7]) / det;
        inv[1] = (a[2] * a[7] - a[1] * a[8]) / det;
        inv[2] = (a[1] * a[5] - a[2] * a[4]) / det;
        inv[3] = (a[5] * a[6] - a[3] * a[8]) / det;
        inv[4] = (a[0] * a[8] - a[2] * a[6]) / det;
        inv[5] = (a[2] * a[3] - a[0] * a[5]) / det;
        inv[6] = (a[3] * a[7] - a[4] * a[6]) / det;
        inv[7] = (a[1] * a[6] - a[0] * a[7]) / det;
        inv[8] = (a[0] * a[4] - a[1] * a[3]) / det;
        // reciprocal rows b_j[k] = 2 pi inv[k][j]
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) g->rlattice[j * 3 + k] = 2.0 * M_PI * inv[k * 3 + j];
        g->volume = fabs(det);
        g->dV = g->volume / (double)N;
        g->prec = precision;
        g->esize = precision == OFDFT_F64 ? sizeof(double) : sizeof(float);
        Geo& geo = g->geo;
        geo.n0 = nr[0];
        geo.n1 = nr[1];
        geo.n2 = nr[2];
        geo.n2h = g->n2h;
        geo.N = N;
        geo.Nc = g->Nc;
        for (int i = 0; i < 9; ++i) {
            geo.b[i] = g->rlattice[i];
            geo.bf[i] = (float)g->rlattice[i];
        }
        for (int d = 0; d < 3; ++d) geo.fv[d] = 1.0 / ((double)nr[d] * (1.0 / (double)nr[d]));
        int dev = 0;
        cudaGetDevice(&dev);
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        g->sms = sms > 0 ? sms : 152;
        // field reductions: up to 8 blocks of 256 threads per SM, fewer on small grids
        // (about 16 points per thread), where block scheduling would dominate
        g->red_blocks = (int)std::max(8LL, std::min((long long)g->sms * 8, (N + 4095) / 4096));
        try {
            OFDFT_CK(cudaMalloc(&g->d_partials, (size_t)g->red_blocks * 32 * sizeof(double)));
            OFDFT_CK(cudaMalloc(&g->d_results, 64 * sizeof(double)));
            OFDFT_CK(cudaMallocHost(&g->h_results, 64 * sizeof(double)));
        } catch (...) {
            ofdft_grid_destroy(g);
            throw;
        }
        *out = g;
    });
}

void ofdft_grid_destroy(ofdft_grid* g) {
    if (!g) return;
    for (auto& kv : g->plans) cufftDestroy(kv.second);
    g->scratch.release_all();
    if (g->d_partials) cudaFree(g->d_partials);
    if (g->d_results) cudaFree(g->d_results);
    if (g->h_results) cudaFreeHost(g->h_results);
    delete g;
}

int ofdft_grid_info(const ofdft_grid* g, int nr[3], double* volume, double* dV, int* precision) {
    return guard([&] {
        OFDFT_REQUIRE(g, "ofdft_grid_info: null grid");
        if (nr)
            for (int d = 0; d < 3; ++d) nr[d] = g->nr[d];
        if (volume) *volume = g->volume;
        if (dV) *dV = g->dV;
        if (precision) *precision = g->prec;
    });
}

int ofdft_fft(ofdft_grid* g, const void* in_real, void* out_cplx, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(g && in_real && out_cplx, "ofdft_fft: null argument");
        cudaStream_t st = (cudaStream_t)s;
        g->exec_r2c(in_real, out_cplx, 1, st);
        long long n2 = g->Nc * 2;
        int nb = blocks_for(n2, 256, g->sms * 8);
        if (g->prec == OFDFT_F64)
            k_scale_copy<double><<<nb, 256, 0, st>>>((double*)out_cplx, (double*)out_cplx, n2, g->dV);
        else
            k_scale_copy<float><<<nb, 256, 0, st>>>((float*)out_cplx, (float*)out_cplx, n2, g->dV);
        OFDFT_LAUNCH_CHECK();
    });
}

int ofdft_ifft(ofdft_grid* g, const void* in_cplx, void* out_real, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(g && in_cplx && out_real, "ofdft_ifft: null argument");
        cudaStream_t st = (cudaStream_t)s;
        // cuFFT's multi-dimensional C2R overwrites its input: copy it to scratch
        // with the 1/(N dV) normalisation folded into the copy.
        void* tmp = g->scratch.get("ifft_in", g->cplx_bytes());
        long long n2 = g->Nc * 2;
        int nb = blocks_for(n2, 256, g->sms * 8);
        double sc = 1.0 / ((double)g->N * g->dV);
        if (g->prec == OFDFT_F64)
            k_scale_copy<double><<<nb, 256, 0, st>>>((const double*)in_cplx, (double*)tmp, n2, sc);
        else
            k_scale_copy<float><<<nb, 256, 0, st>>>((const float*)in_cplx, (float*)tmp, n2, sc);
        OFDFT_LAUNCH_CHECK();
        g->exec_c2r(tmp, out_real, 1, st);
    });
}

static int dot_impl(ofdft_grid* g, const void* a, const void* b, const void* c, double* out, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(g && a && out, "ofdft_dot: null argument");
        cudaStream_t st = (cudaStream_t)s;
        if (g->prec == OFDFT_F64)
            k_dot<double><<<g->red_blocks, RED_THREADS, 0, st>>>((const double*)a, (const double*)b, (const double*)c,
                                                                g->N, g->d_partials);
        else
            k_dot<float><<<g->red_blocks, RED_THREADS, 0, st>>>((const float*)a, (const float*)b, (const float*)c,
                                                               g->N, g->d_partials);
        OFDFT_LAUNCH_CHECK();
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 1, 0ull, g->d_results);
        OFDFT_LAUNCH_CHECK();
        OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        *out = g->h_results[0];
    });
}

int ofdft_dot(ofdft_grid* g, const void* a, const void* b, double* out, ofdft_stream s) {
    return dot_impl(g, a, b, nullptr, out, s);
}

int ofdft_dot3(ofdft_grid* g, const void* a, const void* b, const void* c, double* out, ofdft_stream s) {
    if (!b || !c) {
        ofdft::set_error("ofdft_dot3: null argument");
        return OFDFT_EINVAL;
    }
    return dot_impl(g, a, b, c, out, s);
}

}  // extern "C"
