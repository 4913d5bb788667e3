// Density mixing of OE-SCF (src/dftpy/mixer/mixer.py:8-169, pulay.py:8-120,
// linear.py:4-35): the Pulay history step, the Gram matrix of the residual
// history in one pass over all fields, and the preconditioned mixed density
// (one real-space combination, one batched R2C, one G-space pass, one C2R).
// The small linear solve of the Pulay coefficients stays on the host.
#include "common.cuh"

namespace ofdft {
namespace {

constexpr int kMaxF = OFDFT_MIX_MAXM + 1;

struct FieldList {
    const void* p[kMaxF];
};

struct MixPtrs {
    const void* dn[OFDFT_MIX_MAXM];
    const void* dr[OFDFT_MIX_MAXM];
    double x[OFDFT_MIX_MAXM];
    int ns;
};

// pulay.py:53-56 (r, dn, dr) and :101-102 (the saved density and residual)
template <typename T>
__global__ void k_mix_history(const T* __restrict__ nin, const T* __restrict__ nout, T* prev_n, T* prev_r, T* dn,
                              T* dr, long long N, int first) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const T a = nin[i];
        const T r = nout[i] - a;
        if (!first) {
            dn[i] = a - prev_n[i];
            dr[i] = r - prev_r[i];
        }
        prev_n[i] = a;
        prev_r[i] = r;
    }
}

// Lower triangle of the Gram matrix, row-major (a, b <= a), float64 sums.
template <typename T, int NF>
__global__ void __launch_bounds__(RED_THREADS) k_mix_gram(FieldList f, long long N, double* partials) {
    constexpr int NP = NF * (NF + 1) / 2;
    double acc[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) acc[k] = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        double v[NF];
#pragma unroll
        for (int a = 0; a < NF; ++a) v[a] = (double)((const T*)f.p[a])[i];
        int k = 0;
#pragma unroll
        for (int a = 0; a < NF; ++a)
#pragma unroll
            for (int b = 0; b <= a; ++b) acc[k++] += v[a] * v[b];
    }
    block_sum_store<NP>(acc, partials);
}

// Real-space part of pulay.py:78-92 / linear.py:25-27 and mixer.py:137-139:
// A = nin + sum x_i dn_i, B = coef (resw r + sum x_i dr_i), C = (1 - mc) nin + mc nout,
// r = nout - nin; null history entries add nothing.
template <typename T>
__global__ void k_mix_combine(const T* __restrict__ nin, const T* __restrict__ nout, MixPtrs m, double coef,
                              double mask_coef, double resw, int cutoff, T* A, T* B, T* C, long long N) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const T cf = (T)coef, mc = (T)mask_coef, one = (T)1;
    const bool rw = resw != 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const T a = nin[i], o = nout[i];
        T res = rw ? o - a : (T)0, drho = (T)0;
        bool have_drho = false, have_res = rw;
        for (int k = 0; k < m.ns; ++k) {
            const T xk = (T)m.x[k];
            if (m.dn[k]) {
                const T t = xk * ((const T*)m.dn[k])[i];
                drho = have_drho ? drho + t : t;
                have_drho = true;
            }
            if (m.dr[k]) {
                const T t = xk * ((const T*)m.dr[k])[i];
                res = have_res ? res + t : t;
                have_res = true;
            }
        }
        A[i] = have_drho ? a + drho : a;
        B[i] = res * cf;
        if (cutoff) C[i] = a * (one - mc) + mc * o;
    }
}

// SpecialPrecondition.matrix (mixer.py:28-40, 72-117) as a function of |G|^2.
__device__ inline double pred_matrix(int type, double gg, const double* pc) {
    switch (type) {
        case OFDFT_PRED_KERKER: {
            const double q0 = pc[1] * pc[1];
            return pc[0] * fmin(gg / (gg + q0), pc[2]);
        }
        case OFDFT_PRED_INVERSE_KERKER:
            return gg == 0.0 ? 0.0 : pc[0] * pc[0] / gg + 1.0;
        case OFDFT_PRED_RESTA: {
            if (gg == 0.0) return 1.0;
            const double q0 = pc[1] * pc[1], q = sqrt(gg);
            return (q0 * sin(q * pc[2]) / (pc[0] * q * pc[2]) + gg) / (q0 + gg);
        }
        default:
            return 1.0;
    }
}

struct PredArgs {
    int type;
    double pc[3];
    int cutoff;
    double invN;
};

template <typename C>
__global__ void k_mix_gspace(Geo geo, C* A, const C* B, const C* Cm, const double* gmax, PredArgs p) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const double gm = p.cutoff ? *gmax : 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        const double gg = gsq(geo, i);
        double re, im;
        if (p.cutoff && gg > gm) {
            re = (double)Cm[i].x;
            im = (double)Cm[i].y;
        } else {
            const double m = pred_matrix(p.type, gg, p.pc);
            re = (double)A[i].x + m * (double)B[i].x;
            im = (double)A[i].y + m * (double)B[i].y;
        }
        A[i].x = re * p.invN;
        A[i].y = im * p.invN;
    }
}

// gmax of the high-frequency mask (mixer.py:56-70): 2 ecut, or below ecut = 2
// the largest |G|^2 along the three axes plus 2.  One block.
__global__ void k_mix_gmax(Geo geo, double ecut, double* out) {
    __shared__ double sh[RED_THREADS];
    double m = 0.0;
    for (int i = threadIdx.x; i < geo.n0; i += blockDim.x) m = fmax(m, gsq(geo, (long long)i * geo.n1 * geo.n2h));
    for (int j = threadIdx.x; j < geo.n1; j += blockDim.x) m = fmax(m, gsq(geo, (long long)j * geo.n2h));
    for (int k = threadIdx.x; k < geo.n2h; k += blockDim.x) m = fmax(m, gsq(geo, (long long)k));
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = ecut < 2.0 ? sh[0] + 2.0 : 2.0 * ecut;
}

template <typename T>
void history_t(ofdft_grid* g, const void* nin, const void* nout, void* pn, void* pr, void* dn, void* dr, int first,
               cudaStream_t st) {
    const int nb = blocks_for(g->N, 256, g->sms * 8);
    k_mix_history<T><<<nb, 256, 0, st>>>((const T*)nin, (const T*)nout, (T*)pn, (T*)pr, (T*)dn, (T*)dr, g->N,
                                         first);
    OFDFT_LAUNCH_CHECK();
}

template <typename T, int NF>
void gram_launch(ofdft_grid* g, const FieldList& f, double* partials, cudaStream_t st) {
    k_mix_gram<T, NF><<<g->red_blocks, RED_THREADS, 0, st>>>(f, g->N, partials);
}

template <typename T>
void gram_t(ofdft_grid* g, const void* const* fields, int nf, double* gram, cudaStream_t st) {
    FieldList f{};
    for (int a = 0; a < nf; ++a) f.p[a] = fields[a];
    const int np = nf * (nf + 1) / 2;
    double* partials = (double*)g->scratch.get("mix_partials", (size_t)g->red_blocks * np * sizeof(double));
    double* res = (double*)g->scratch.get("mix_results", 64 * sizeof(double));
    switch (nf) {
        case 1: gram_launch<T, 1>(g, f, partials, st); break;
        case 2: gram_launch<T, 2>(g, f, partials, st); break;
        case 3: gram_launch<T, 3>(g, f, partials, st); break;
        case 4: gram_launch<T, 4>(g, f, partials, st); break;
        case 5: gram_launch<T, 5>(g, f, partials, st); break;
        case 6: gram_launch<T, 6>(g, f, partials, st); break;
        case 7: gram_launch<T, 7>(g, f, partials, st); break;
        case 8: gram_launch<T, 8>(g, f, partials, st); break;
        default: gram_launch<T, 9>(g, f, partials, st); break;
    }
    OFDFT_LAUNCH_CHECK();
    reduce_finalize<<<1, RED_THREADS, 0, st>>>(partials, g->red_blocks, np, 0ull, res);
    OFDFT_LAUNCH_CHECK();
    double tri[kMaxF * (kMaxF + 1) / 2];
    OFDFT_CK(cudaMemcpyAsync(tri, res, np * sizeof(double), cudaMemcpyDeviceToHost, st));
    OFDFT_CK(cudaStreamSynchronize(st));
    int k = 0;
    for (int a = 0; a < nf; ++a)
        for (int b = 0; b <= a; ++b, ++k) gram[a * nf + b] = gram[b * nf + a] = tri[k];
}

template <typename T>
void density_t(ofdft_grid* g, const void* nin, const void* nout, const ofdft_mix_args* a, void* out, cudaStream_t st) {
    using C = typename Cplx<T>::type;
    const long long N = g->N;
    const int batch = a->cutoff ? 3 : 2;
    T* real = (T*)g->scratch.get("mix_real", (size_t)batch * g->real_bytes());
    C* cplx = (C*)g->scratch.get("mix_cplx", (size_t)batch * g->cplx_bytes());
    double* gmax = (double*)g->scratch.get("mix_gmax", sizeof(double));
    MixPtrs m{};
    m.ns = a->ns;
    for (int k = 0; k < a->ns; ++k) {
        m.dn[k] = a->dn[k];
        m.dr[k] = a->dr[k];
        m.x[k] = a->x[k];
    }
    const int nb = blocks_for(N, 256, g->sms * 8);
    k_mix_combine<T><<<nb, 256, 0, st>>>((const T*)nin, (const T*)nout, m, a->coef, a->mask_coef, a->resw, a->cutoff, real,
                                         real + N, a->cutoff ? real + 2 * N : nullptr, N);
    OFDFT_LAUNCH_CHECK();
    g->exec_r2c(real, cplx, batch, st);
    if (a->cutoff) {
        k_mix_gmax<<<1, RED_THREADS, 0, st>>>(g->geo, a->predecut, gmax);
        OFDFT_LAUNCH_CHECK();
    }
    PredArgs p{};
    p.type = a->predtype;
    for (int k = 0; k < 3; ++k) p.pc[k] = a->predcoef[k];
    p.cutoff = a->cutoff;
    p.invN = 1.0 / (double)N;
    const int gb = blocks_for(g->Nc, 256, g->sms * 8);
    k_mix_gspace<C><<<gb, 256, 0, st>>>(g->geo, cplx, cplx + g->Nc, a->cutoff ? cplx + 2 * g->Nc : nullptr, gmax, p);
    OFDFT_LAUNCH_CHECK();
    g->exec_c2r(cplx, out, 1, st);
}

}  // namespace
}  // namespace ofdft

using namespace ofdft;

extern "C" {

int ofdft_mix_history(ofdft_grid* g, const void* nin, const void* nout, void* prev_n, void* prev_r, void* dn, void* dr,
                      int first, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(g && nin && nout && prev_n && prev_r, "ofdft_mix_history: null argument");
        OFDFT_REQUIRE(first || (dn && dr), "ofdft_mix_history: dn and dr are required after the first step");
        if (g->esize == 8)
            history_t<double>(g, nin, nout, prev_n, prev_r, dn, dr, first, (cudaStream_t)s);
        else
            history_t<float>(g, nin, nout, prev_n, prev_r, dn, dr, first, (cudaStream_t)s);
    });
}

int ofdft_mix_gram(ofdft_grid* g, const void* const* fields, int nf, double* gram, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(g && fields && gram, "ofdft_mix_gram: null argument");
        OFDFT_REQUIRE(nf >= 1 && nf <= kMaxF, "ofdft_mix_gram: nf = %d outside 1..%d", nf, kMaxF);
        for (int a = 0; a < nf; ++a) OFDFT_REQUIRE(fields[a], "ofdft_mix_gram: field %d is null", a);
        if (g->esize == 8)
            gram_t<double>(g, fields, nf, gram, (cudaStream_t)s);
        else
            gram_t<float>(g, fields, nf, gram, (cudaStream_t)s);
    });
}

int ofdft_mix_density(ofdft_grid* g, const void* nin, const void* nout, const ofdft_mix_args* a, void* out,
                      ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(g && nin && nout && a && out, "ofdft_mix_density: null argument");
        OFDFT_REQUIRE(out != nin && out != nout, "ofdft_mix_density: out aliases an input");
        OFDFT_REQUIRE(a->ns >= 0 && a->ns <= OFDFT_MIX_MAXM, "ofdft_mix_density: ns = %d outside 0..%d", a->ns,
                      OFDFT_MIX_MAXM);
        OFDFT_REQUIRE(a->predtype >= OFDFT_PRED_NONE && a->predtype <= OFDFT_PRED_RESTA,
                      "ofdft_mix_density: unknown predtype %d", a->predtype);
        if (g->esize == 8)
            density_t<double>(g, nin, nout, a, out, (cudaStream_t)s);
        else
            density_t<float>(g, nin, nout, a, out, (cudaStream_t)s);
    });
}

}  // extern "C"
