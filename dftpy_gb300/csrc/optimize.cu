// Density optimisation on phi = sqrt(rho) (Optimization.optimize_rho,
// src/dftpy/optimization/optimization.py:283-525) with the line search of
// scipy's line_search_wolfe1 (math_utils.py:37-52): the MINPACK-2 routine
// dcsrch/dcstep of More and Thuente (ACM TOMS 20, 1994), restated here.
// All field work stays on the device; only scalars (energies, dot products,
// line-search state) live on the host.
#include "common.cuh"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <vector>

using namespace ofdft;

namespace {

// ------------------------------------------------------------ line search
// dcstep: safeguarded cubic/quadratic step and bracket update.
void dcstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp, double fp,
            double dp, bool& brackt, double stpmin, double stpmax) {
    auto sgn = [](double v) { return (double)((v > 0) - (v < 0)); };
    const double sgnd = sgn(dp) * sgn(dx);
    double stpf;
    if (fp > fx) {
        // higher function value: minimum bracketed; cubic unless the quadratic is closer
        double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
        double s = std::max(std::fabs(theta), std::max(std::fabs(dx), std::fabs(dp)));
        double gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
        if (stp < stx) gamma = -gamma;
        double p = (gamma - dx) + theta;
        double q = ((gamma - dx) + gamma) + dp;
        double r = p / q;
        double stpc = stx + r * (stp - stx);
        double stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx);
        stpf = std::fabs(stpc - stx) <= std::fabs(stpq - stx) ? stpc : stpc + (stpq - stpc) / 2.0;
        brackt = true;
    } else if (sgnd < 0.0) {
        // lower value, derivatives of opposite sign: bracketed; cubic if farther than secant
        double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
        double s = std::max(std::fabs(theta), std::max(std::fabs(dx), std::fabs(dp)));
        double gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
        if (stp > stx) gamma = -gamma;
        double p = (gamma - dp) + theta;
        double q = ((gamma - dp) + gamma) + dx;
        double r = p / q;
        double stpc = stp + r * (stx - stp);
        double stpq = stp + (dp / (dp - dx)) * (stx - stp);
        stpf = std::fabs(stpc - stp) > std::fabs(stpq - stp) ? stpc : stpq;
        brackt = true;
    } else if (std::fabs(dp) < std::fabs(dx)) {
        // lower value, same-sign derivatives of decreasing magnitude
        double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
        double s = std::max(std::fabs(theta), std::max(std::fabs(dx), std::fabs(dp)));
        double gamma = s * std::sqrt(std::max(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
        if (stp > stx) gamma = -gamma;
        double p = (gamma - dp) + theta;
        double q = (gamma + (dx - dp)) + gamma;
        double r = p / q;
        double stpc;
        if (r < 0 && gamma != 0) stpc = stp + r * (stx - stp);
        else if (stp > stx) stpc = stpmax;
        else stpc = stpmin;
        double stpq = stp + (dp / (dp - dx)) * (stx - stp);
        if (brackt) {
            stpf = std::fabs(stpc - stp) < std::fabs(stpq - stp) ? stpc : stpq;
            if (stp > stx) stpf = std::min(stp + 0.66 * (sty - stp), stpf);
            else stpf = std::max(stp + 0.66 * (sty - stp), stpf);
        } else {
            stpf = std::fabs(stpc - stp) > std::fabs(stpq - stp) ? stpc : stpq;
            stpf = std::min(std::max(stpf, stpmin), stpmax);
        }
    } else {
        // lower value, same-sign derivatives not decreasing
        if (brackt) {
            double theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp;
            double s = std::max(std::fabs(theta), std::max(std::fabs(dy), std::fabs(dp)));
            double gamma = s * std::sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
            if (stp > sty) gamma = -gamma;
            double p = (gamma - dp) + theta;
            double q = ((gamma - dp) + gamma) + dy;
            double r = p / q;
            stpf = stp + r * (sty - stp);
        } else {
            stpf = stp > stx ? stpmax : stpmin;
        }
    }
    if (fp > fx) {
        sty = stp;
        fy = fp;
        dy = dp;
    } else {
        if (sgnd < 0) {
            sty = stx;
            fy = fx;
            dy = dx;
        }
        stx = stp;
        fx = fp;
        dx = dp;
    }
    stp = stpf;
}

enum Task { FG, CONV, WARN, ERR };

struct Dcsrch {
    double ftol, gtol, xtol, stpmin, stpmax;
    bool brackt = false;
    int stage = 1;
    double ginit = 0, gtest = 0, gx = 0, gy = 0, finit = 0, fx = 0, fy = 0, stx = 0, sty = 0, stmin = 0, stmax = 0,
           width = 0, width1 = 0;

    Task start(double& stp, double f, double g) {
        if (stp < stpmin || stp > stpmax || g >= 0 || ftol < 0 || gtol < 0 || xtol < 0 || stpmin < 0 ||
            stpmax < stpmin)
            return ERR;
        brackt = false;
        stage = 1;
        finit = f;
        ginit = g;
        gtest = ftol * ginit;
        width = stpmax - stpmin;
        width1 = width / 0.5;
        stx = 0.0;
        fx = finit;
        gx = ginit;
        sty = 0.0;
        fy = finit;
        gy = ginit;
        stmin = 0;
        stmax = stp + 4.0 * stp;
        return FG;
    }

    Task iterate(double& stp, double f, double g) {
        const double ftest = finit + stp * gtest;
        if (stage == 1 && f <= ftest && g >= 0) stage = 2;
        Task task = FG;
        if (brackt && (stp <= stmin || stp >= stmax)) task = WARN;
        if (brackt && stmax - stmin <= xtol * stmax) task = WARN;
        if (stp == stpmax && f <= ftest && g <= gtest) task = WARN;
        if (stp == stpmin && (f > ftest || g >= gtest)) task = WARN;
        if (f <= ftest && std::fabs(g) <= gtol * -ginit) task = CONV;
        if (task == WARN || task == CONV) return task;
        if (stage == 1 && f <= fx && f > ftest) {
            // modified function psi(stp) = f - stp*gtest in the first stage
            double fm = f - stp * gtest, fxm = fx - stx * gtest, fym = fy - sty * gtest;
            double gm = g - gtest, gxm = gx - gtest, gym = gy - gtest;
            dcstep(stx, fxm, gxm, sty, fym, gym, stp, fm, gm, brackt, stmin, stmax);
            fx = fxm + stx * gtest;
            fy = fym + sty * gtest;
            gx = gxm + gtest;
            gy = gym + gtest;
        } else {
            dcstep(stx, fx, gx, sty, fy, gy, stp, f, g, brackt, stmin, stmax);
        }
        if (brackt) {
            if (std::fabs(sty - stx) >= 0.66 * width1) stp = stx + 0.5 * (sty - stx);
            width1 = width;
            width = std::fabs(sty - stx);
        }
        if (brackt) {
            stmin = std::min(stx, sty);
            stmax = std::max(stx, sty);
        } else {
            stmin = stp + 1.1 * (stp - stx);
            stmax = stp + 4.0 * (stp - stx);
        }
        stp = std::min(std::max(stp, stpmin), stpmax);
        if ((brackt && (stp <= stmin || stp >= stmax)) || (brackt && stmax - stmin <= xtol * stmax)) stp = stx;
        return FG;
    }
};

// Line search on the directional derivative alone (no energy comparisons), for
// stages whose energies carry float32 round-off larger than the decreases near
// convergence.  The rotation phi cos(theta) + p sin(theta) repeats the density
// with period pi, so the search stays in (0, amax] with amax well below pi/2:
// from stp0, steps grow by secant extrapolation of phi' (at most 4x per step)
// while phi' < 0, then regula falsi between the bracketing steps (a bisection
// when the secant lands within 1% of an end) until |phi'| <= c2 |phi'(0)|.  The
// accepted step is the last one evaluated.  Returns false when phi'(0) >= 0, when
// phi' is still negative at amax or when no bracket is found in maxiter
// evaluations.  Not in the reference (whose line search is scipy's MINPACK-2 on
// the energy); meant for a stage that starts near the ground state.
template <class Phi>
bool grad_search(Phi&& phi, double g0, double stp0, double c2, double amax, int maxiter, double& stp, double& f,
                 double& g, int& nfev) {
    nfev = 0;
    if (!(g0 < 0.0)) return false;
    const double tol = c2 * std::fabs(g0);
    double lo = 0.0, glo = g0, hi = 0.0, ghi = 0.0;
    bool bracket = false;
    double t = std::min(stp0, amax);
    while (nfev < maxiter) {
        double ft, gt;
        phi(t, ft, gt);
        ++nfev;
        stp = t;
        f = ft;
        g = gt;
        if (!std::isfinite(gt)) return false;
        if (std::fabs(gt) <= tol) return true;
        if (gt < 0.0) {
            const double tp = lo, gp = glo;
            lo = t;
            glo = gt;
            if (!bracket) {
                if (t >= amax) return false;
                // root of the secant of phi' through the last two points, at most 4x further
                double tn = (gt < gp) ? 4.0 * t : t - gt * (t - tp) / (gt - gp);
                tn = std::min(std::max(tn, 1.5 * t), 4.0 * t);
                t = std::min(tn, amax);
                continue;
            }
        } else {
            hi = t;
            ghi = gt;
            bracket = true;
        }
        const double w = hi - lo;
        t = lo - glo * w / (ghi - glo);
        if (!(t > lo + 0.01 * w && t < hi - 0.01 * w)) t = 0.5 * (lo + hi);
    }
    return bracket;
}

// scalar_search_wolfe1 semantics: start at stp0, at most maxiter dcsrch calls;
// returns false when no acceptable step is found.  phi(stp, f, g) evaluates.
template <class Phi>
bool wolfe1(Phi&& phi, double f0, double g0, double stp0, double c1, double c2, double amax, double amin,
            double xtol, int maxiter, double& stp, double& f, double& g, int& nfev) {
    Dcsrch d;
    d.ftol = c1;
    d.gtol = c2;
    d.xtol = xtol;
    d.stpmin = amin;
    d.stpmax = amax;
    stp = stp0;
    f = f0;
    g = g0;
    nfev = 0;
    Task t = d.start(stp, f, g);
    if (t == ERR) return false;
    for (int it = 0; it < maxiter; ++it) {
        if (it > 0) t = d.iterate(stp, f, g);
        if (!std::isfinite(stp)) return false;
        if (t != FG) return t == CONV;
        phi(stp, f, g);
        ++nfev;
    }
    return false;
}

// ------------------------------------------------------------- field ops
// Element arithmetic runs in the grid precision T (GB300 runs float64 at a
// small fraction of the float32 rate); sums run per thread in RunSum<T> and
// across threads in float64.
template <typename T>
struct RunSum;
template <>
struct RunSum<double> {
    double s = 0.0;
    __device__ void add(double x) { s += x; }
    __device__ double get() const { return s; }
};
template <>
struct RunSum<float> {
    float s = 0.0f, c = 0.0f;
    __device__ void add(float x) {  // Kahan-compensated
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ double get() const { return (double)s - (double)c; }
};

// Rounded operations spelled out (no contraction left to the compiler), so that
// the single-system and the batched kernels give the same bits.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// b0 x0 + b1 x1 + b2 x2 (absent terms skipped)
template <typename T>
__device__ __forceinline__ T lin3(T b0, const T* x0, T b1, const T* x1, T b2, const T* x2, long long i) {
    T v = mul_rn(b0, x0[i]);
    if (x1) v = fma_rn(b1, x1[i], v);
    if (x2) v = fma_rn(b2, x2[i], v);
    return v;
}
// phi cos + p sin
template <typename T>
__device__ __forceinline__ T rot(T phi, T p, T c, T s) {
    return fma_rn(phi, c, mul_rn(p, s));
}
// V nphi (p cos - phi sin)
template <typename T>
__device__ __forceinline__ T dth_term(T V, T nphi, T p, T phi, T c, T s) {
    return mul_rn(mul_rn(V, nphi), fma_rn(p, c, -mul_rn(phi, s)));
}

template <typename T>
__global__ void k_lincomb(long long n, T* out, double a0, const T* x0, double a1, const T* x1, double a2,
                          const T* x2) {
    const T b0 = (T)a0, b1 = (T)a1, b2 = (T)a2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = lin3(b0, x0, b1, x1, b2, x2, i);
}

// get_direction_CG with CG-CD (math_utils.py:341-342, 347): beta is the field
// -(r*r)/s, so p = -r + (-(r*r)/s) d point by point
template <typename T>
__global__ void k_cg_cd(long long n, T* p, const T* r, const T* d, double s) {
    const T ss = (T)s;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const T ri = r[i];
        const T b = -mul_rn(ri, ri) / ss;
        p[i] = fma_rn(b, d[i], -ri);
    }
}

// sqrt(rho), 1e-300 where rho <= 0 (0 in float32, where 1e-300 underflows)
template <typename T>
__device__ inline T phi_floor();
template <>
__device__ inline double phi_floor<double>() { return 1e-300; }
template <>
__device__ inline float phi_floor<float>() { return 0.0f; }

template <typename T>
__global__ void k_phi_init(long long n, const T* rho, T* phi) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const T r = rho[i];
        phi[i] = r > (T)0 ? sqrt(r) : phi_floor<T>();
    }
}

// out = x^2 (the density of a phi)
template <typename T>
__global__ void k_square(long long n, const T* x, T* out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const T v = x[i];
        out[i] = mul_rn(v, v);
    }
}

// newphi = phi cos + p sin, rho = newphi^2
template <typename T>
__global__ void k_rotate(long long n, const T* phi, const T* p, double c, double s, T* newphi, T* rho) {
    const T cw = (T)c, sw = (T)s;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const T v = rot(phi[i], p[i], cw, sw);
        newphi[i] = v;
        rho[i] = mul_rn(v, v);
    }
}

// out = (V - mu) phi
template <typename T>
__global__ void k_resid(long long n, const T* V, double mu, const T* phi, T* out) {
    const T m = (T)mu;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = mul_rn(sub_rn(V[i], m), phi[i]);
}

// Ap = ((V1 - mu) phi1 - res0) / eps
template <typename T>
__global__ void k_tn_ap(long long n, const T* V1, double mu, const T* phi1, const T* res0, double eps, T* Ap) {
    const T m = (T)mu, ep = (T)eps;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        Ap[i] = ((V1[i] - m) * phi1[i] - res0[i]) / ep;
}

// sum V * newphi * (p cos - phi sin)
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_dtheta(long long n, const T* V, const T* nphi, const T* p,
                                                        const T* phi, double c, double s, double* partials) {
    const T cw = (T)c, sw = (T)s;
    RunSum<T> sum;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        sum.add(dth_term(V[i], nphi[i], p[i], phi[i], cw, sw));
    double acc[1] = {sum.get()};
    block_sum_store<1>(acc, partials);
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_dot2(long long n, const T* a, const T* b, double* partials) {
    RunSum<T> sum;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        sum.add(mul_rn(a[i], b[i]));
    double acc[1] = {sum.get()};
    block_sum_store<1>(acc, partials);
}

}  // namespace

// grid of an evaluator (the evaluator struct lives in total.cu)
ofdft_grid* e_grid(ofdft_eval* e);
// an evaluation enqueued without waiting, and its energies after a synchronisation (total.cu)
void eval_enqueue(ofdft_eval* e, const void* rho, void* v_out, unsigned calc, cudaStream_t st);
void eval_collect(ofdft_eval* e, double* energies);
ofdft_batch_eval* batch_eval_open(int n, ofdft_eval** evs, void* const* rho, void* const* v, cudaStream_t st);
void batch_eval_close(ofdft_batch_eval* b);
void batch_eval_enqueue(ofdft_batch_eval* b, void* const* rho, void* const* v, const unsigned char* act,
                        cudaStream_t st);
double batch_eval_energy(const ofdft_batch_eval* b, int s);
bool eval_capturable(const ofdft_eval* e);

namespace {

template <typename T>
struct Opt {
    ofdft_eval* e;
    ofdft_grid* g;
    cudaStream_t st;
    long long N;
    int eb;
    // Work fields live in the grid's scratch under "opt_" names, so repeated
    // optimisations on one grid allocate them once.

    T* buf(const char* name) { return (T*)g->scratch.get(std::string("opt_") + name, g->real_bytes()); }
    double finish() {
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 1, 0ull, g->d_results + 32);
        OFDFT_LAUNCH_CHECK();
        OFDFT_CK(cudaMemcpyAsync(g->h_results + 32, g->d_results + 32, sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        return g->h_results[32];
    }
    double dot(const T* a, const T* b) {
        k_dot2<T><<<g->red_blocks, RED_THREADS, 0, st>>>(N, a, b, g->d_partials);
        OFDFT_LAUNCH_CHECK();
        return finish();
    }
    double dtheta(const T* V, const T* nphi, const T* p, const T* phi, double c, double s) {
        k_dtheta<T><<<g->red_blocks, RED_THREADS, 0, st>>>(N, V, nphi, p, phi, c, s, g->d_partials);
        OFDFT_LAUNCH_CHECK();
        return finish();
    }
    void lincomb(T* out, double a0, const T* x0, double a1 = 0, const T* x1 = nullptr, double a2 = 0,
                 const T* x2 = nullptr) {
        k_lincomb<T><<<eb, 256, 0, st>>>(N, out, a0, x0, a1, x1, a2, x2);
        OFDFT_LAUNCH_CHECK();
    }
    void copy(T* out, const T* in) { OFDFT_CK(cudaMemcpyAsync(out, in, g->real_bytes(), cudaMemcpyDeviceToDevice, st)); }
    double eval(const T* rho, T* V, unsigned calc) {
        double E[OFDFT_NE];
        int rc = ofdft_eval_compute(e, rho, V, calc, E, st);
        if (rc != OFDFT_OK) throw Error{rc};
        return E[OFDFT_E_TOTAL];
    }
    // OrthogonalNormalization (optimization.py:205-226): p -= (p.phi/Ne) phi; |p|^2 = Ne
    double orth_norm(T* p, const T* phi) {
        const double dV = g->dV;
        double Ne = dot(phi, phi) * dV;
        double f = dot(p, phi) * dV / Ne;
        lincomb(p, 1.0, p, -f, phi);
        double pN = dot(p, p) * dV;
        double theta = std::sqrt(pN / Ne);
        lincomb(p, std::sqrt(Ne / pN), p);
        return theta;
    }
};

template <typename T>
void optimize_t(ofdft_eval* e, T* rho_io, const ofdft_opt_options& o, ofdft_opt_result& res, T* v_out,
                cudaStream_t st) {
    Opt<T> op;
    op.e = e;
    op.g = e_grid(e);
    op.st = st;
    op.N = op.g->N;
    op.eb = blocks_for(op.N, 256, op.g->sms * 16);
    ofdft_grid* g = op.g;
    const double dV = g->dV;
    const long long N = op.N;
    T* phi = op.buf("phi");
    T* V = op.buf("V");
    T* rsd = op.buf("res");
    T* p = op.buf("p");
    T* nphi = op.buf("nphi");
    T* nrho = op.buf("nrho");
    T* nV = op.buf("nV");
    // phi = sqrt(rho) with rho <= 0 -> 1e-300, renormalised (optimization.py:305-315)
    k_phi_init<T><<<op.eb, 256, 0, st>>>(N, rho_io, phi);
    OFDFT_LAUNCH_CHECK();
    double srho = 0.0;
    ofdft_dot(g, rho_io, nullptr, &srho, st);
    double sphi = op.dot(phi, phi);
    op.lincomb(phi, std::sqrt(srho / sphi), phi);
    T* rho = op.buf("rho");
    k_square<T><<<op.eb, 256, 0, st>>>(N, phi, rho);
    OFDFT_LAUNCH_CHECK();
    double E = op.eval(rho, V, OFDFT_CALC_E | OFDFT_CALC_V);
    // get_chemical_potential (optimization.py:542-544): mu = int(V rho) / N
    double Nel = 0.0;
    ofdft_dot(g, rho, nullptr, &Nel, st);
    Nel *= dV;
    double mu = op.dot(V, rho) * dV / Nel;
    k_resid<T><<<op.eb, 256, 0, st>>>(N, V, mu, phi, rsd);
    OFDFT_LAUNCH_CHECK();
    std::vector<double> Ehist{E};
    // history buffers
    T* res_prev = op.buf("res_prev");
    T* dir_prev = op.buf("dir_prev");
    bool have_res_prev = false, have_dir_prev = false;
    struct Pair {
        T* s;
        T* y;
        double rho;
    };
    std::deque<Pair> lb;
    int pool_i = 0;
    auto lb_buf = [&]() {
        std::string nm = "lb" + std::to_string(pool_i++);
        return op.buf(nm.c_str());
    };
    // TN work
    T* dvec = (o.method == OFDFT_OPT_TN) ? op.buf("tn_d") : nullptr;
    T* rr = (o.method == OFDFT_OPT_TN) ? op.buf("tn_r") : nullptr;
    T* pp = (o.method == OFDFT_OPT_TN) ? op.buf("tn_p") : nullptr;
    T* phi1 = (o.method == OFDFT_OPT_TN) ? op.buf("tn_phi1") : nullptr;
    T* rho1 = (o.method == OFDFT_OPT_TN) ? op.buf("tn_rho1") : nullptr;
    T* V1 = (o.method == OFDFT_OPT_TN) ? op.buf("tn_V1") : nullptr;
    T* Ap = (o.method == OFDFT_OPT_TN) ? op.buf("tn_Ap") : nullptr;
    T* best = (o.method == OFDFT_OPT_TN) ? op.buf("tn_best") : nullptr;
    T* old_phi = op.buf("old_phi");
    // finite-difference step of the Hessian products: 1e-9 as in the reference in
    // float64; float32 fields cannot resolve it, so the mixed path uses 1e-4
    const double eps = sizeof(T) == 8 ? 1.0e-9 : 1.0e-4;
    int converged = 2, it = 0, nfev = 1;
    double last_stp = 0.0;    // the derivative search's last accepted step
    double last_scale = 0.0;  // ls_start: the last accepted step over its direction's length (0: none yet)
    for (it = 1; it < o.maxiter; ++it) {
        if (o.method == OFDFT_OPT_DIIS) {
            // The reference's DIIS (optimization.py:327-333, :429-441, :471-485):
            // 'Scaling' leaves p = -r as it is; a step phi + 0.1 p renormalised to
            // the current electron count, evaluated for V only; then a second step
            // phi + 0.1 p from the new residual, whose renormalisation factor is
            // rho.N / rho.integral() of the same fresh field, i.e. 1, so it is not
            // renormalised; that density's E and V end the iteration.
            op.lincomb(p, -1.0, rsd);
            op.lincomb(nphi, 1.0, phi, 0.1, p);
            k_square<T><<<op.eb, 256, 0, st>>>(N, nphi, nrho);
            OFDFT_LAUNCH_CHECK();
            double sn = 0.0;
            ofdft_dot(g, nrho, nullptr, &sn, st);
            const double norm = Nel / (sn * dV);
            op.lincomb(nrho, norm, nrho);
            op.lincomb(nphi, std::sqrt(norm), nphi);
            op.eval(nrho, nV, OFDFT_CALC_V);
            op.copy(old_phi, phi);
            op.copy(phi, nphi);
            k_square<T><<<op.eb, 256, 0, st>>>(N, phi, rho);
            OFDFT_LAUNCH_CHECK();
            ofdft_dot(g, rho, nullptr, &Nel, st);
            Nel *= dV;
            mu = op.dot(nV, rho) * dV / Nel;
            k_resid<T><<<op.eb, 256, 0, st>>>(N, nV, mu, phi, rsd);
            OFDFT_LAUNCH_CHECK();
            op.lincomb(p, -1.0, rsd);
            op.lincomb(phi, 1.0, phi, 0.1, p);
            k_square<T><<<op.eb, 256, 0, st>>>(N, phi, rho);
            OFDFT_LAUNCH_CHECK();
            E = op.eval(rho, V, OFDFT_CALC_E | OFDFT_CALC_V);
            nfev += 2;
            ofdft_dot(g, rho, nullptr, &Nel, st);
            Nel *= dV;
            mu = op.dot(V, rho) * dV / Nel;
            k_resid<T><<<op.eb, 256, 0, st>>>(N, V, mu, phi, rsd);
            OFDFT_LAUNCH_CHECK();
            Ehist.push_back(E);
            const double resN = op.dot(rsd, rsd) * dV;
            res.dP = resN;
            if (o.verbose)
                fprintf(stderr, "%-8d%-24.12E%-16.6E%-16.6E%-8d\n", it, E, Ehist[Ehist.size() - 1] - Ehist[Ehist.size() - 2],
                        resN, 1);
            bool conv = false;
            if ((int)Ehist.size() - 1 >= o.ncheck) {
                conv = true;
                for (int i = 0; i < o.ncheck; ++i)
                    if (std::fabs(Ehist[Ehist.size() - 2 - i] - E) > o.econv) conv = false;
            }
            if (conv) {
                converged = 0;
                break;
            }
            continue;
        }
        // ---- direction
        if (o.method == OFDFT_OPT_TN) {
            // get_direction_TN (optimization.py:92-148)
            OFDFT_CK(cudaMemsetAsync(dvec, 0, g->real_bytes(), st));
            op.lincomb(rr, -1.0, rsd);
            op.copy(pp, rr);
            double r0 = op.dot(rr, rr);
            const double rconv = r0 * 0.1;
            bool have_best = false;
            std::vector<double> rl{1e10};
            bool use_best = false;
            for (int k = 0; k < o.maxfun; ++k) {
                op.lincomb(phi1, 1.0, phi, eps, pp);
                k_square<T><<<op.eb, 256, 0, st>>>(N, phi1, rho1);
                OFDFT_LAUNCH_CHECK();
                op.eval(rho1, V1, OFDFT_CALC_V);
                nfev++;
                k_tn_ap<T><<<op.eb, 256, 0, st>>>(N, V1, mu, phi1, rsd, eps, Ap);
                OFDFT_LAUNCH_CHECK();
                double pAp = op.dot(pp, Ap);
                if (pAp < 0.0) {
                    if (k == 0) op.lincomb(dvec, r0 / pAp, pp);
                    break;
                }
                double alpha = r0 / pAp;
                op.lincomb(dvec, 1.0, dvec, alpha, pp);
                op.lincomb(rr, 1.0, rr, -alpha, Ap);
                double r1 = op.dot(rr, rr);
                double rmin = *std::min_element(rl.begin(), rl.end());
                if (r1 < rmin) {
                    op.copy(best, dvec);
                    have_best = true;
                }
                rl.push_back(r1);
                if (r1 < rconv) break;
                double rmin_prev = *std::min_element(rl.begin(), rl.end() - 1);
                if (r1 > 1000 * rmin_prev) {
                    use_best = true;
                    break;
                } else if (k > 10 && std::fabs(r0 - r1) < 0.1 * r0) {
                    use_best = true;
                    break;
                }
                double beta = r1 / r0;
                r0 = r1;
                op.lincomb(pp, 1.0, rr, beta, pp);
            }
            if (use_best) {
                if (have_best) op.copy(dvec, best);
                else OFDFT_CK(cudaMemsetAsync(dvec, 0, g->real_bytes(), st));
            }
            op.copy(p, dvec);
        } else if (o.method == OFDFT_OPT_LBFGS) {
            // get_direction_LBFGS (optimization.py:150-171): the first loop skips i = 0
            T* q = op.buf("lb_q");
            op.lincomb(q, -1.0, rsd);
            const int m = (int)lb.size();
            std::vector<double> al(m, 0.0);
            for (int i = m - 1; i > 0; --i) {
                double a = lb[i].rho * op.dot(lb[i].s, q);
                al[i] = a;
                op.lincomb(q, 1.0, q, -a, lb[i].y);
            }
            if (o.h0 == 0.0) {
                double gamma = m < 1 ? 1.0 : op.dot(lb[m - 1].s, lb[m - 1].y) / op.dot(lb[m - 1].y, lb[m - 1].y);
                op.lincomb(p, gamma, q);
            } else {
                op.lincomb(p, o.h0, q);
            }
            for (int i = 0; i < m; ++i) {
                double b = lb[i].rho * op.dot(lb[i].y, p);
                op.lincomb(p, 1.0, p, al[i] - b, lb[i].s);
            }
        } else if (o.method == OFDFT_OPT_GD) {
            // get_direction_GD (math_utils.py:352-354)
            op.lincomb(p, -1.0, rsd);
        } else {
            // get_direction_CG (math_utils.py:326-349): beta from the last two
            // residuals and the last direction; -r on the first iteration
            if (have_res_prev && have_dir_prev) {
                T* dr = op.buf("cg_dr");
                op.lincomb(dr, 1.0, rsd, -1.0, res_prev);
                double beta = 0.0;
                switch (o.method) {
                    case OFDFT_OPT_CGHS: beta = op.dot(rsd, dr) / op.dot(dir_prev, dr); break;
                    case OFDFT_OPT_CGPR: beta = std::max(op.dot(rsd, dr) / op.dot(res_prev, res_prev), 0.0); break;
                    case OFDFT_OPT_CGDY: beta = op.dot(rsd, rsd) / op.dot(dir_prev, dr); break;
                    case OFDFT_OPT_CGLS: beta = op.dot(rsd, dr) / op.dot(dir_prev, res_prev); break;
                    case OFDFT_OPT_CGFR: beta = op.dot(rsd, rsd) / op.dot(res_prev, res_prev); break;
                    default: break;
                }
                if (o.method == OFDFT_OPT_CGCD) {
                    k_cg_cd<T><<<op.eb, 256, 0, st>>>(N, p, rsd, dir_prev, op.dot(dir_prev, res_prev));
                    OFDFT_LAUNCH_CHECK();
                } else {
                    op.lincomb(p, -1.0, rsd, beta, dir_prev);
                }
            } else {
                op.lincomb(p, -1.0, rsd);
            }
        }
        // the direction's length before normalisation: the quasi-Newton (L-BFGS) or
        // Newton (TN) step along it, the first trial step when ls_start = 1
        double theta0 = op.orth_norm(p, phi);
        bool natural = o.ls_start == 1 && (o.method == OFDFT_OPT_LBFGS || o.method == OFDFT_OPT_TN);
        if (op.dtheta(V, phi, p, phi, 1.0, 0.0) * 2.0 > 0) {
            // uphill: steepest descent (optimization.py:373-380)
            op.lincomb(p, -1.0, rsd);
            op.orth_norm(p, phi);
            natural = false;
        }
        // ---- line search on theta (ValueAndDerivative, optimization.py:228-280)
        double lastE = NAN, last_theta = NAN;
        auto phi_fn = [&](double th, double& f, double& gd) {
            const double c = std::cos(th), s = std::sin(th);
            k_rotate<T><<<op.eb, 256, 0, st>>>(N, phi, p, c, s, nphi, nrho);
            OFDFT_LAUNCH_CHECK();
            f = op.eval(nrho, nV, OFDFT_CALC_E | OFDFT_CALC_V);
            gd = 2.0 * op.dtheta(nV, nphi, p, phi, c, s) * dV;
            lastE = f;
            last_theta = th;
        };
        const double g0 = 2.0 * op.dtheta(V, phi, p, phi, 1.0, 0.0) * dV;
        double stp, fnew, gnew;
        int nls = 0;
        // first trial step: the reference's 1.0 for the energy search; twice the last accepted
        // step (0.1 at first) for the derivative search; with ls_start = 1, once a step has been
        // accepted, the direction's length theta0 times the last accepted step's ratio to its
        // direction's length (the quasi-Newton step with its scale corrected), within each
        // search's bound (pi or pi/4)
        const bool nat = natural && theta0 > 0.0 && std::isfinite(theta0) && last_scale > 0.0;
        const double s0w = nat ? std::min(theta0 * last_scale, M_PI) : 1.0;
        const double s0g = nat ? std::min(theta0 * last_scale, M_PI / 4) : (last_stp > 0.0 ? 2.0 * last_stp : 0.1);
        bool ok = o.ls_grad ? grad_search(phi_fn, g0, s0g, o.c2, M_PI / 4, 20, stp, fnew, gnew, nls)
                            : wolfe1(phi_fn, E, g0, s0w, o.c1, o.c2, M_PI, 0.0, o.xtol, 100, stp, fnew, gnew, nls);
        if (ok) last_stp = stp;
        if (ok && natural && theta0 > 0.0 && std::isfinite(theta0)) last_scale = stp / theta0;
        nfev += nls;
        if (!ok || nls == 0 || stp != last_theta) {
            converged = 1;  // "Line-Search Failed" (optimization.py:444-448)
            break;
        }
        // ---- accept
        op.copy(old_phi, phi);
        op.copy(phi, nphi);
        op.copy(V, nV);
        E = lastE;
        k_square<T><<<op.eb, 256, 0, st>>>(N, phi, rho);
        OFDFT_LAUNCH_CHECK();
        ofdft_dot(g, rho, nullptr, &Nel, st);
        Nel *= dV;
        mu = op.dot(V, rho) * dV / Nel;
        op.copy(res_prev, rsd);
        have_res_prev = true;
        k_resid<T><<<op.eb, 256, 0, st>>>(N, V, mu, phi, rsd);
        OFDFT_LAUNCH_CHECK();
        if (o.method == OFDFT_OPT_LBFGS) {
            // LBFGS.update (math_utils.py:307-325): at most maxcor+1 pairs
            Pair pr;
            if ((int)lb.size() > o.maxcor) {
                pr = lb.front();
                lb.pop_front();
            } else {
                pr.s = lb_buf();
                pr.y = lb_buf();
            }
            op.lincomb(pr.s, 1.0, phi, -1.0, old_phi);
            op.lincomb(pr.y, 1.0, rsd, -1.0, res_prev);
            pr.rho = 1.0 / op.dot(pr.y, pr.s);
            lb.push_back(pr);
        }
        Ehist.push_back(E);
        const double resN = op.dot(rsd, rsd) * dV;
        res.dP = resN;
        if (o.verbose)
            fprintf(stderr, "%-8d%-24.12E%-16.6E%-16.6E%-8d\n", it, E, Ehist[Ehist.size() - 1] - Ehist[Ehist.size() - 2],
                    resN, nls);
        if (o.pconv > 0.0 && resN <= o.pconv) {  // the residual criterion (off by default)
            converged = 0;
            break;
        }
        // check_converge (optimization.py:527-540)
        bool conv = false;
        if ((int)Ehist.size() - 1 >= o.ncheck) {
            conv = true;
            for (int i = 0; i < o.ncheck; ++i)
                if (std::fabs(Ehist[Ehist.size() - 2 - i] - E) > o.econv) conv = false;
        }
        if (conv) {
            converged = 0;
            break;
        }
        op.copy(dir_prev, p);
        have_dir_prev = true;
    }
    // rho_io <- phi^2; the potential of the last accepted evaluation is that of rho_io
    k_square<T><<<op.eb, 256, 0, st>>>(N, phi, rho_io);
    OFDFT_LAUNCH_CHECK();
    if (v_out) OFDFT_CK(cudaMemcpyAsync(v_out, V, g->real_bytes(), cudaMemcpyDeviceToDevice, st));
    OFDFT_CK(cudaStreamSynchronize(st));
    res.converged = converged;
    // iterations run, as the reference counts them: maxiter - 1 when the budget ran out
    res.niter = std::min(it, o.maxiter - 1);
    res.nfev = nfev;
    res.energy = E;
    res.mu = mu;
    if (converged != 0) res.dP = op.dot(rsd, rsd) * dV;
}

// ------------------------------------------------------------------------
// Lockstep L-BFGS over a batch of independent systems (uneven grids allowed).
//
// Every system runs the algorithm of optimize_t (L-BFGS branch) on its own
// fields, with its own line search; the systems advance together, so each
// vector operation is one launch over all systems (a block-to-system map in
// device memory, per-system coefficients in the kernel arguments) and each
// round of scalars is one device-to-host copy and one stream synchronisation
// for the whole batch.  Evaluations stay per system (their cuFFT plans are per
// grid) but are enqueued back to back and collected after one synchronisation.
// The arithmetic of every operation, reductions included, is that of the
// single-system optimiser, so each system's result is the same as a solve on
// its own.

constexpr int kBatchMax = 128;  // systems per batch (per-system arguments travel in the launch)
constexpr int kBF = 48;         // field slots per system

enum BField {
    BF_RHOIO = 0,
    BF_PHI,
    BF_V,
    BF_RSD,
    BF_P,
    BF_NPHI,
    BF_NRHO,
    BF_NV,
    BF_OLDPHI,
    BF_RESPREV,
    BF_Q,
    BF_RHO,
    BF_LB0  // L-BFGS pair buffers from here on
};

template <typename T>
struct BTab {
    T* f[kBF];
    long long N;
    int red_blocks;  // the system grid's reduction block count
    int boff;        // first block of the system in a reduction launch
    int eoff, eb;    // first block and block count in an elementwise launch
    double dV;
};

// per-system coefficients and the active mask, passed by value
struct BArgs {
    double c[kBatchMax][3];
    unsigned char act[kBatchMax];
};

// Device-resident scalars of the batch, kSc rows of kBatchMax: dot results,
// L-BFGS coefficients and the per-system coefficients of the next field update,
// so that the two-loop recursion and the normalisations run without the host.
constexpr int kHist = kBF;  // alpha_i of the two-loop, by pair position
enum ScRow { SC_D0 = 0, SC_D1, SC_NE, SC_MU, SC_NEL, SC_C0, SC_C1, SC_C2, SC_TH0, SC_AL0, SC_LBRHO0 = SC_AL0 + kHist,
             kSc = SC_LBRHO0 + kBF };

__device__ __forceinline__ double* scrow(double* sc, int r) { return sc + (size_t)r * kBatchMax; }

// one thread per system; op selects the scalar update (the same float64
// operations, in the same order, as the host code of optimize_t)
enum ScOp { OP_AL, OP_B, OP_LBRHO, OP_ORTH_F, OP_ORTH_N, OP_MU };
template <typename T>
__global__ void k_bscalar(const BTab<T>* __restrict__ tab, BArgs a, double* sc, int S, int op, int i, int slot) {
    const int s = threadIdx.x;
    if (s >= S || !a.act[s]) return;
    const double dV = tab[s].dV;
    const double d0 = scrow(sc, SC_D0)[s], d1 = scrow(sc, SC_D1)[s];
    double c0 = 1.0, c1 = 0.0;
    switch (op) {
        case OP_AL: {  // alpha_i = rho_i (s_i . q); q -= alpha_i y_i
            const double al = __dmul_rn(scrow(sc, SC_LBRHO0 + slot)[s], d0);
            scrow(sc, SC_AL0 + i)[s] = al;
            c1 = -al;
            break;
        }
        case OP_B:  // beta = rho_i (y_i . p); p += (alpha_i - beta) s_i
            c1 = __dsub_rn(scrow(sc, SC_AL0 + i)[s], __dmul_rn(scrow(sc, SC_LBRHO0 + slot)[s], d0));
            break;
        case OP_LBRHO:  // rho = 1 / (y . s)
            scrow(sc, SC_LBRHO0 + slot)[s] = 1.0 / d0;
            return;
        case OP_ORTH_F: {  // Ne = (phi.phi) dV; p -= ((p.phi) dV / Ne) phi
            const double ne = __dmul_rn(d0, dV);
            scrow(sc, SC_NE)[s] = ne;
            c1 = -(__dmul_rn(d1, dV) / ne);
            break;
        }
        case OP_ORTH_N: {  // p *= sqrt(Ne / ((p.p) dV)); the direction's length sqrt((p.p) dV / Ne)
            const double pn = __dmul_rn(d0, dV), ne = scrow(sc, SC_NE)[s];
            scrow(sc, SC_TH0)[s] = sqrt(pn / ne);
            c0 = sqrt(ne / pn);
            break;
        }
        case OP_MU: {  // Nel = sum(rho) dV; mu = (V.rho) dV / Nel
            const double nel = __dmul_rn(d0, dV);
            const double mu = __dmul_rn(d1, dV) / nel;
            scrow(sc, SC_NEL)[s] = nel;
            scrow(sc, SC_MU)[s] = mu;
            c0 = mu;
            break;
        }
    }
    scrow(sc, SC_C0)[s] = c0;
    scrow(sc, SC_C1)[s] = c1;
    scrow(sc, SC_C2)[s] = 0.0;
}

template <typename T>
__global__ void k_blincomb(const BTab<T>* __restrict__ tab, const int* __restrict__ esys, BArgs a, int o, int x0,
                           int x1, int x2) {
    const int s = esys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const T b0 = (T)a.c[s][0], b1 = (T)a.c[s][1], b2 = (T)a.c[s][2];
    T* out = t.f[o];
    const T* X0 = t.f[x0];
    const T* X1 = x1 >= 0 ? t.f[x1] : nullptr;
    const T* X2 = x2 >= 0 ? t.f[x2] : nullptr;
    const long long stride = (long long)t.eb * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.eoff) * blockDim.x + threadIdx.x; i < t.N; i += stride)
        out[i] = lin3(b0, X0, b1, X1, b2, X2, i);
}

template <typename T>
__global__ void k_bsquare(const BTab<T>* __restrict__ tab, const int* __restrict__ esys, BArgs a, int x, int o) {
    const int s = esys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const long long stride = (long long)t.eb * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.eoff) * blockDim.x + threadIdx.x; i < t.N; i += stride) {
        const T v = t.f[x][i];
        t.f[o][i] = mul_rn(v, v);
    }
}

template <typename T>
__global__ void k_bphi_init(const BTab<T>* __restrict__ tab, const int* __restrict__ esys, BArgs a) {
    const int s = esys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const long long stride = (long long)t.eb * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.eoff) * blockDim.x + threadIdx.x; i < t.N; i += stride) {
        const T r = t.f[BF_RHOIO][i];
        t.f[BF_PHI][i] = r > (T)0 ? sqrt(r) : phi_floor<T>();
    }
}

// nphi = phi cos + p sin, nrho = nphi^2 (c[s] = {cos, sin})
template <typename T>
__global__ void k_brotate(const BTab<T>* __restrict__ tab, const int* __restrict__ esys, BArgs a) {
    const int s = esys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const T cw = (T)a.c[s][0], sw = (T)a.c[s][1];
    const long long stride = (long long)t.eb * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.eoff) * blockDim.x + threadIdx.x; i < t.N; i += stride) {
        const T v = rot(t.f[BF_PHI][i], t.f[BF_P][i], cw, sw);
        t.f[BF_NPHI][i] = v;
        t.f[BF_NRHO][i] = mul_rn(v, v);
    }
}

// rsd = (V - mu) phi (c[s][0] = mu)
template <typename T>
__global__ void k_bresid(const BTab<T>* __restrict__ tab, const int* __restrict__ esys, BArgs a) {
    const int s = esys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const T m = (T)a.c[s][0];
    const long long stride = (long long)t.eb * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.eoff) * blockDim.x + threadIdx.x; i < t.N; i += stride)
        t.f[BF_RSD][i] = mul_rn(sub_rn(t.f[BF_V][i], m), t.f[BF_PHI][i]);
}

// k_blincomb with the coefficients read from the device scalars
template <typename T>
__global__ void k_blincomb_dc(const BTab<T>* __restrict__ tab, const int* __restrict__ esys, BArgs a,
                              const double* __restrict__ sc, int o, int x0, int x1) {
    const int s = esys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const T b0 = (T)sc[SC_C0 * kBatchMax + s], b1 = (T)sc[SC_C1 * kBatchMax + s];
    T* out = t.f[o];
    const T* X0 = t.f[x0];
    const T* X1 = x1 >= 0 ? t.f[x1] : nullptr;
    const long long stride = (long long)t.eb * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.eoff) * blockDim.x + threadIdx.x; i < t.N; i += stride)
        out[i] = lin3(b0, X0, b1, X1, (T)0, (const T*)nullptr, i);
}

// rsd = (V - mu) phi with mu from the device scalars
template <typename T>
__global__ void k_bresid_dc(const BTab<T>* __restrict__ tab, const int* __restrict__ esys, BArgs a,
                            const double* __restrict__ sc) {
    const int s = esys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const T m = (T)sc[SC_MU * kBatchMax + s];
    const long long stride = (long long)t.eb * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.eoff) * blockDim.x + threadIdx.x; i < t.N; i += stride)
        t.f[BF_RSD][i] = mul_rn(sub_rn(t.f[BF_V][i], m), t.f[BF_PHI][i]);
}

// sum a*b per system, accumulated as k_dot2 does
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_bdot2(const BTab<T>* __restrict__ tab, const int* __restrict__ bsys,
                                                       BArgs a, int xa, int xb, double* partials) {
    const int s = bsys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const T* A = t.f[xa];
    const T* B = t.f[xb];
    RunSum<T> sum;
    const long long stride = (long long)t.red_blocks * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.boff) * blockDim.x + threadIdx.x; i < t.N; i += stride)
        sum.add(mul_rn(A[i], B[i]));
    double acc[1] = {sum.get()};
    block_sum_store_at<1>(acc, partials, blockIdx.x);
}

// sum a per system in float64, accumulated as ofdft_dot (k_dot) does
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_bsum(const BTab<T>* __restrict__ tab, const int* __restrict__ bsys,
                                                      BArgs a, int xa, double* partials) {
    const int s = bsys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const T* A = t.f[xa];
    double v[1] = {0.0};
    const long long stride = (long long)t.red_blocks * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.boff) * blockDim.x + threadIdx.x; i < t.N; i += stride)
        v[0] += (double)A[i];
    block_sum_store_at<1>(v, partials, blockIdx.x);
}

// sum V * nphi * (p cos - phi sin) per system, as k_dtheta (c[s] = {cos, sin}; fields given)
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_bdtheta(const BTab<T>* __restrict__ tab, const int* __restrict__ bsys,
                                                         BArgs a, int xV, int xnphi, double* partials) {
    const int s = bsys[blockIdx.x];
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    const T cw = (T)a.c[s][0], sw = (T)a.c[s][1];
    const T *V = t.f[xV], *nphi = t.f[xnphi], *p = t.f[BF_P], *phi = t.f[BF_PHI];
    RunSum<T> sum;
    const long long stride = (long long)t.red_blocks * blockDim.x;
    for (long long i = (long long)(blockIdx.x - t.boff) * blockDim.x + threadIdx.x; i < t.N; i += stride)
        sum.add(dth_term(V[i], nphi[i], p[i], phi[i], cw, sw));
    double acc[1] = {sum.get()};
    block_sum_store_at<1>(acc, partials, blockIdx.x);
}

// one block per system: its partials reduced with the tree of reduce_finalize
template <typename T>
__global__ void k_bfinalize(const BTab<T>* __restrict__ tab, BArgs a, const double* __restrict__ partials,
                            double* out) {
    const int s = blockIdx.x;
    if (!a.act[s]) return;
    const BTab<T>& t = tab[s];
    __shared__ double sh[RED_THREADS];
    double x = 0.0;
    for (int b = threadIdx.x; b < t.red_blocks; b += blockDim.x) x += partials[t.boff + b];
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[s] = sh[0];
}

template <typename T>
struct Batch {
    int S = 0;
    std::vector<ofdft_eval*> e;
    std::vector<ofdft_grid*> g;
    cudaStream_t st = nullptr;
    std::vector<BTab<T>> h_tab;
    BTab<T>* d_tab = nullptr;
    int *d_bsys = nullptr, *d_esys = nullptr;
    int nb_red = 0, nb_el = 0;
    double* d_part = nullptr;
    double* d_out = nullptr;   // kMaxRound rows of S scalars
    double* h_out = nullptr;   // pinned mirror
    int rows = 0;              // scalar rows queued since the last sync
    static constexpr int kMaxRound = 8;
    BArgs args{};

    // evaluations of a round are spread over worker streams (forked from and
    // joined back to st), so that the small kernels of many systems overlap
    static constexpr int kStreams = 16;
    std::vector<cudaStream_t> ws;
    std::vector<cudaEvent_t> wev;
    cudaEvent_t fork_ev = nullptr;

    // the line-search evaluation (nrho -> nV) of each system, captured once as
    // a CUDA graph and replayed: one launch instead of a dozen per evaluation
    std::vector<cudaGraphExec_t> gexec;

    ~Batch() {
        for (cudaGraphExec_t x : gexec)
            if (x) cudaGraphExecDestroy(x);
        for (cudaStream_t w : ws) cudaStreamDestroy(w);
        for (cudaEvent_t v : wev) cudaEventDestroy(v);
        if (fork_ev) cudaEventDestroy(fork_ev);
        cudaFree(d_tab);
        cudaFree(d_bsys);
        cudaFree(d_esys);
        cudaFree(d_part);
        cudaFree(d_out);
        cudaFree(d_sc);
        cudaFreeHost(h_out);
    }

    T* field(int s, const char* name) {
        return (T*)g[s]->scratch.get(std::string("opt_") + name, g[s]->real_bytes());
    }

    void setup(int nsys, ofdft_eval** evs, void** rho_io, int npairs, cudaStream_t stream) {
        S = nsys;
        st = stream;
        e.assign(evs, evs + S);
        g.resize(S);
        h_tab.resize(S);
        std::vector<int> bsys, esys;
        for (int s = 0; s < S; ++s) {
            g[s] = e_grid(e[s]);
            BTab<T>& t = h_tab[s];
            memset(&t, 0, sizeof(t));
            t.N = g[s]->N;
            t.red_blocks = g[s]->red_blocks;
            t.boff = (int)bsys.size();
            for (int b = 0; b < t.red_blocks; ++b) bsys.push_back(s);
            t.eb = blocks_for(t.N, 256, g[s]->sms * 16);
            t.eoff = (int)esys.size();
            for (int b = 0; b < t.eb; ++b) esys.push_back(s);
            t.f[BF_RHOIO] = (T*)rho_io[s];
            t.dV = g[s]->dV;
            static const char* names[] = {"", "phi", "V", "res", "p", "nphi", "nrho", "nV", "old_phi", "res_prev",
                                          "lb_q", "rho"};
            for (int f = 1; f < BF_LB0; ++f) t.f[f] = field(s, names[f]);
            for (int k = 0; k < npairs; ++k) t.f[BF_LB0 + k] = field(s, ("lb" + std::to_string(k)).c_str());
        }
        nb_red = (int)bsys.size();
        nb_el = (int)esys.size();
        OFDFT_CK(cudaMalloc(&d_tab, S * sizeof(BTab<T>)));
        OFDFT_CK(cudaMalloc(&d_bsys, nb_red * sizeof(int)));
        OFDFT_CK(cudaMalloc(&d_esys, nb_el * sizeof(int)));
        OFDFT_CK(cudaMalloc(&d_part, (size_t)nb_red * sizeof(double)));
        OFDFT_CK(cudaMalloc(&d_out, (size_t)kMaxRound * S * sizeof(double)));
        OFDFT_CK(cudaMallocHost(&h_out, (size_t)kMaxRound * S * sizeof(double)));
        OFDFT_CK(cudaMalloc(&d_sc, (size_t)kSc * kBatchMax * sizeof(double)));
        OFDFT_CK(cudaMemsetAsync(d_sc, 0, (size_t)kSc * kBatchMax * sizeof(double), st));
        OFDFT_CK(cudaMemcpyAsync(d_tab, h_tab.data(), S * sizeof(BTab<T>), cudaMemcpyHostToDevice, st));
        OFDFT_CK(cudaMemcpyAsync(d_bsys, bsys.data(), nb_red * sizeof(int), cudaMemcpyHostToDevice, st));
        OFDFT_CK(cudaMemcpyAsync(d_esys, esys.data(), nb_el * sizeof(int), cudaMemcpyHostToDevice, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        const int nw = std::min(S, kStreams);
        ws.resize(nw);
        wev.resize(nw);
        for (int k = 0; k < nw; ++k) {
            OFDFT_CK(cudaStreamCreateWithFlags(&ws[k], cudaStreamNonBlocking));
            OFDFT_CK(cudaEventCreateWithFlags(&wev[k], cudaEventDisableTiming));
        }
        OFDFT_CK(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
        gexec.assign(S, nullptr);
    }
    // the line-search evaluation of system s on its worker stream, captured on
    // first use (the evaluation's buffers and plans exist by then: the starting
    // evaluation ran uncaptured)
    void eval_ls(int s) {
        cudaStream_t w = worker(s);
        if (!gexec[s] && eval_capturable(e[s])) {
            cudaGraph_t graph = nullptr;
            OFDFT_CK(cudaStreamBeginCapture(w, cudaStreamCaptureModeThreadLocal));
            try {
                eval_enqueue(e[s], h_tab[s].f[BF_NRHO], h_tab[s].f[BF_NV], OFDFT_CALC_E | OFDFT_CALC_V, w);
            } catch (...) {
                cudaStreamEndCapture(w, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            OFDFT_CK(cudaStreamEndCapture(w, &graph));
            const cudaError_t rc = cudaGraphInstantiate(&gexec[s], graph, 0);
            cudaGraphDestroy(graph);
            OFDFT_CK(rc);
        }
        if (gexec[s]) OFDFT_CK(cudaGraphLaunch(gexec[s], w));
        else eval_enqueue(e[s], h_tab[s].f[BF_NRHO], h_tab[s].f[BF_NV], OFDFT_CALC_E | OFDFT_CALC_V, w);
    }
    // fork: worker streams wait for everything queued on st so far
    void fork() {
        OFDFT_CK(cudaEventRecord(fork_ev, st));
        for (cudaStream_t w : ws) OFDFT_CK(cudaStreamWaitEvent(w, fork_ev, 0));
    }
    cudaStream_t worker(int s) const { return ws[s % (int)ws.size()]; }
    // join: st waits for everything queued on the worker streams
    void join() {
        for (size_t k = 0; k < ws.size(); ++k) {
            OFDFT_CK(cudaEventRecord(wev[k], ws[k]));
            OFDFT_CK(cudaStreamWaitEvent(st, wev[k], 0));
        }
    }

    void coef(int s, double c0, double c1 = 0.0, double c2 = 0.0) {
        args.c[s][0] = c0;
        args.c[s][1] = c1;
        args.c[s][2] = c2;
    }
    // elementwise launches over the systems marked active in args
    void lincomb(int o, int x0, int x1 = -1, int x2 = -1) {
        k_blincomb<T><<<nb_el, 256, 0, st>>>(d_tab, d_esys, args, o, x0, x1, x2);
        OFDFT_LAUNCH_CHECK();
    }
    void copy(int o, int x) {
        for (int s = 0; s < S; ++s) coef(s, 1.0);
        lincomb(o, x);
    }
    void square(int x, int o) {
        k_bsquare<T><<<nb_el, 256, 0, st>>>(d_tab, d_esys, args, x, o);
        OFDFT_LAUNCH_CHECK();
    }
    // reductions: each queues one row of S scalars, read after sync()
    int finish_row() {
        OFDFT_REQUIRE(rows < kMaxRound, "batched optimiser: too many scalars queued in one round");
        k_bfinalize<T><<<S, RED_THREADS, 0, st>>>(d_tab, args, d_part, d_out + (size_t)rows * S);
        OFDFT_LAUNCH_CHECK();
        return rows++;
    }
    int dot(int xa, int xb) {
        k_bdot2<T><<<nb_red, RED_THREADS, 0, st>>>(d_tab, d_bsys, args, xa, xb, d_part);
        OFDFT_LAUNCH_CHECK();
        return finish_row();
    }
    int sum(int xa) {
        k_bsum<T><<<nb_red, RED_THREADS, 0, st>>>(d_tab, d_bsys, args, xa, d_part);
        OFDFT_LAUNCH_CHECK();
        return finish_row();
    }
    int dtheta(int xV, int xnphi) {
        k_bdtheta<T><<<nb_red, RED_THREADS, 0, st>>>(d_tab, d_bsys, args, xV, xnphi, d_part);
        OFDFT_LAUNCH_CHECK();
        return finish_row();
    }
    // queues device scalar row `row` for the host, like a reduction's row
    int queue_sc(int row) {
        OFDFT_REQUIRE(rows < kMaxRound, "batched optimiser: too many scalars queued in one round");
        OFDFT_CK(cudaMemcpyAsync(d_out + (size_t)rows * S, d_sc + (size_t)row * kBatchMax, (size_t)S * sizeof(double),
                                 cudaMemcpyDeviceToDevice, st));
        return rows++;
    }
    // device-only reductions: the result stays in device scalar row `row`
    double* d_sc = nullptr;  // kSc x kBatchMax
    void fin_dev(int row) {
        k_bfinalize<T><<<S, RED_THREADS, 0, st>>>(d_tab, args, d_part, d_sc + (size_t)row * kBatchMax);
        OFDFT_LAUNCH_CHECK();
    }
    void dot_dev(int xa, int xb, int row) {
        k_bdot2<T><<<nb_red, RED_THREADS, 0, st>>>(d_tab, d_bsys, args, xa, xb, d_part);
        OFDFT_LAUNCH_CHECK();
        fin_dev(row);
    }
    void sum_dev(int xa, int row) {
        k_bsum<T><<<nb_red, RED_THREADS, 0, st>>>(d_tab, d_bsys, args, xa, d_part);
        OFDFT_LAUNCH_CHECK();
        fin_dev(row);
    }
    void scalar(int op, int i = 0, int slot = 0) {
        k_bscalar<T><<<1, kBatchMax, 0, st>>>(d_tab, args, d_sc, S, op, i, slot);
        OFDFT_LAUNCH_CHECK();
    }
    void lincomb_dc(int o, int x0, int x1 = -1) {
        k_blincomb_dc<T><<<nb_el, 256, 0, st>>>(d_tab, d_esys, args, d_sc, o, x0, x1);
        OFDFT_LAUNCH_CHECK();
    }
    // OrthogonalNormalization (optimization.py:205-226) without the host
    void orth_norm_dev() {
        dot_dev(BF_PHI, BF_PHI, SC_D0);
        dot_dev(BF_P, BF_PHI, SC_D1);
        scalar(OP_ORTH_F);
        lincomb_dc(BF_P, BF_P, BF_PHI);
        dot_dev(BF_P, BF_P, SC_D0);
        scalar(OP_ORTH_N);
        lincomb_dc(BF_P, BF_P);
    }
    // one device-to-host copy of the queued rows and one synchronisation
    void sync() {
        if (rows) OFDFT_CK(cudaMemcpyAsync(h_out, d_out, (size_t)rows * S * sizeof(double), cudaMemcpyDeviceToHost, st));
        const auto t0 = std::chrono::steady_clock::now();
        OFDFT_CK(cudaStreamSynchronize(st));
        wait_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        ++syncs;
        rows = 0;
    }
    double wait_s = 0.0, enqueue_s = 0.0;  // host time waiting in sync() / enqueueing evaluations
    long long syncs = 0, evals = 0;
    double at(int row, int s) const { return h_out[(size_t)row * S + s]; }
    void set_active(const std::vector<char>& act) {
        for (int s = 0; s < S; ++s) args.act[s] = act[s] ? 1 : 0;
    }
};

template <typename T>
void optimize_batch_t(int S, ofdft_eval** evs, void** rho_io, const ofdft_opt_options& o, const double* econv,
                      ofdft_opt_result* res, void** v_out, cudaStream_t st) {
    OFDFT_REQUIRE(o.method == OFDFT_OPT_LBFGS, "ofdft_optimize_batch: only L-BFGS is batched");
    OFDFT_REQUIRE(o.pconv == 0.0 && o.ls_grad == 0,
                  "ofdft_optimize_batch: the residual criterion and the derivative line search are not batched");
    OFDFT_REQUIRE(o.maxcor >= 0 && 2 * (o.maxcor + 1) <= kBF - BF_LB0, "ofdft_optimize_batch: maxcor too large");
    Batch<T> b;
    const int npairs = 2 * (o.maxcor + 1);
    b.setup(S, evs, rho_io, npairs, st);
    std::vector<double> dV(S), E(S), mu(S), Nel(S);
    for (int s = 0; s < S; ++s) dV[s] = b.g[s]->dV;
    std::vector<char> run(S, 1);  // still iterating
    std::vector<int> conv(S, 2), niter(S, 0), nfev(S, 1);
    std::vector<std::vector<double>> Ehist(S);
    std::vector<double> dP(S, 0.0);
    std::vector<char> accepted_any(S, 0);  // mu then lives in the device scalars
    auto active = [&](const std::vector<char>& m) { b.set_active(m); };
    auto any = [](const std::vector<char>& m) { return std::any_of(m.begin(), m.end(), [](char c) { return c != 0; }); };
    // persistent mode: one cooperative launch per round for every active system
    struct PbOwner {
        ofdft_batch_eval* p = nullptr;
        ~PbOwner() {
            if (p) batch_eval_close(p);
        }
    } pb;
    if (o.batch_persistent) {
        std::vector<void*> r(S), v(S);
        for (int s = 0; s < S; ++s) {
            r[s] = b.h_tab[s].f[BF_RHOIO];
            v[s] = b.h_tab[s].f[BF_V];
        }
        pb.p = batch_eval_open(S, evs, r.data(), v.data(), st);
    }
    auto evaluate = [&](const std::vector<char>& m, int xrho, int xV) {
        const auto t0 = std::chrono::steady_clock::now();
        if (pb.p) {
            std::vector<void*> r(S), v(S);
            std::vector<unsigned char> act(S);
            for (int s = 0; s < S; ++s) {
                r[s] = b.h_tab[s].f[xrho];
                v[s] = b.h_tab[s].f[xV];
                act[s] = m[s] ? 1 : 0;
                if (m[s]) ++b.evals;
            }
            batch_eval_enqueue(pb.p, r.data(), v.data(), act.data(), st);
            b.enqueue_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            return;
        }
        b.fork();
        for (int s = 0; s < S; ++s)
            if (m[s]) {
                if (xrho == BF_NRHO && xV == BF_NV) b.eval_ls(s);
                else eval_enqueue(b.e[s], b.h_tab[s].f[xrho], b.h_tab[s].f[xV], OFDFT_CALC_E | OFDFT_CALC_V,
                                  b.worker(s));
                ++b.evals;
            }
        b.join();
        b.enqueue_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    };
    const auto t_start = std::chrono::steady_clock::now();
    auto collect = [&](const std::vector<char>& m, std::vector<double>& out) {
        if (pb.p) {
            for (int s = 0; s < S; ++s)
                if (m[s]) out[s] = batch_eval_energy(pb.p, s);
            return;
        }
        double En[OFDFT_NE];
        for (int s = 0; s < S; ++s)
            if (m[s]) {
                eval_collect(b.e[s], En);
                out[s] = En[OFDFT_E_TOTAL];
            }
    };
    // ---- start (optimize_t: phi = sqrt(rho) renormalised, first evaluation, mu, residual)
    active(run);
    k_bphi_init<T><<<b.nb_el, 256, 0, st>>>(b.d_tab, b.d_esys, b.args);
    OFDFT_LAUNCH_CHECK();
    {
        const int rr = b.sum(BF_RHOIO), rp = b.dot(BF_PHI, BF_PHI);
        b.sync();
        for (int s = 0; s < S; ++s) b.coef(s, std::sqrt(b.at(rr, s) / b.at(rp, s)));
    }
    b.lincomb(BF_PHI, BF_PHI);
    b.square(BF_PHI, BF_RHO);
    evaluate(run, BF_RHO, BF_V);
    {
        const int rn = b.sum(BF_RHO), rm = b.dot(BF_V, BF_RHO);
        b.sync();
        collect(run, E);
        for (int s = 0; s < S; ++s) {
            Nel[s] = b.at(rn, s) * dV[s];
            mu[s] = b.at(rm, s) * dV[s] / Nel[s];
            b.coef(s, mu[s]);
            Ehist[s].push_back(E[s]);
        }
    }
    k_bresid<T><<<b.nb_el, 256, 0, st>>>(b.d_tab, b.d_esys, b.args);
    OFDFT_LAUNCH_CHECK();
    // L-BFGS pairs: the same slots and history length for every running system
    struct Pair {
        int s, y;
    };
    std::deque<Pair> lb;
    int pool_i = 0;
    std::vector<double> last_scale(S, 0.0);  // ls_start: optimize_t's last_scale per system
    for (int it = 1; it < o.maxiter && any(run); ++it) {
        for (int s = 0; s < S; ++s)
            if (run[s]) niter[s] = it;
        active(run);
        // ---- direction: get_direction_LBFGS (optimization.py:150-171), first loop skips i = 0;
        // the dot products and coefficients stay on the device
        for (int s = 0; s < S; ++s) b.coef(s, -1.0);
        b.lincomb(BF_Q, BF_RSD);
        const int m = (int)lb.size();
        for (int i = m - 1; i > 0; --i) {
            b.dot_dev(lb[i].s, BF_Q, SC_D0);
            b.scalar(OP_AL, i, lb[i].s - BF_LB0);
            b.lincomb_dc(BF_Q, BF_Q, lb[i].y);
        }
        OFDFT_REQUIRE(o.h0 != 0.0, "ofdft_optimize_batch: h0 = 0 is not batched");
        for (int s = 0; s < S; ++s) b.coef(s, o.h0);
        b.lincomb(BF_P, BF_Q);
        for (int i = 0; i < m; ++i) {
            b.dot_dev(lb[i].y, BF_P, SC_D0);
            b.scalar(OP_B, i, lb[i].s - BF_LB0);
            b.lincomb_dc(BF_P, BF_P, lb[i].s);
        }
        b.orth_norm_dev();
        // ls_start: the direction's length before normalisation (optimize_t's theta0)
        const int rth = o.ls_start == 1 ? b.queue_sc(SC_TH0) : -1;
        // uphill: steepest descent (optimization.py:373-380); otherwise this dtheta is g0
        std::vector<double> g0(S, 0.0), theta0(S, 0.0);
        std::vector<char> natural(S, 0);
        {
            for (int s = 0; s < S; ++s) b.coef(s, 1.0, 0.0);
            const int r = b.dtheta(BF_V, BF_PHI);
            b.sync();
            std::vector<char> up(S, 0);
            for (int s = 0; s < S; ++s) {
                up[s] = run[s] && b.at(r, s) * 2.0 > 0;
                g0[s] = 2.0 * b.at(r, s) * dV[s];
                if (rth >= 0) theta0[s] = b.at(rth, s);
                natural[s] = rth >= 0 && run[s] && !up[s];
            }
            if (any(up)) {
                active(up);
                for (int s = 0; s < S; ++s) b.coef(s, -1.0);
                b.lincomb(BF_P, BF_RSD);
                b.orth_norm_dev();
                for (int s = 0; s < S; ++s) b.coef(s, 1.0, 0.0);
                const int r2 = b.dtheta(BF_V, BF_PHI);
                b.sync();
                for (int s = 0; s < S; ++s)
                    if (up[s]) g0[s] = 2.0 * b.at(r2, s) * dV[s];
                active(run);
            }
        }
        // ---- line search on theta: scalar_search_wolfe1 per system, evaluations batched
        std::vector<Dcsrch> ls(S);
        std::vector<double> stp(S, 1.0), f(S), gd(S), lastE(S, NAN), last_theta(S, NAN);
        std::vector<int> nls(S, 0), lsit(S, 0);
        std::vector<char> searching(S, 0), ok(S, 0);
        std::vector<Task> task(S, FG);
        for (int s = 0; s < S; ++s) {
            if (!run[s]) continue;
            // first trial step as optimize_t's (ls_start: the scaled direction length once known)
            if (natural[s] && theta0[s] > 0.0 && std::isfinite(theta0[s]) && last_scale[s] > 0.0)
                stp[s] = std::min(theta0[s] * last_scale[s], M_PI);
            Dcsrch& d = ls[s];
            d.ftol = o.c1;
            d.gtol = o.c2;
            d.xtol = o.xtol;
            d.stpmin = 0.0;
            d.stpmax = M_PI;
            f[s] = E[s];
            gd[s] = g0[s];
            task[s] = d.start(stp[s], f[s], gd[s]);
            searching[s] = task[s] != ERR;
            ok[s] = 0;
        }
        while (any(searching)) {
            // advance each state machine to its next trial step (wolfe1)
            std::vector<char> need(S, 0);
            for (int s = 0; s < S; ++s) {
                if (!searching[s]) continue;
                if (lsit[s] >= 100) {  // wolfe1's maxiter: no further dcsrch call
                    searching[s] = 0;
                    continue;
                }
                if (lsit[s] > 0) task[s] = ls[s].iterate(stp[s], f[s], gd[s]);
                if (!std::isfinite(stp[s])) {
                    searching[s] = 0;
                    continue;
                }
                if (task[s] != FG) {
                    searching[s] = 0;
                    ok[s] = task[s] == CONV;
                    continue;
                }
                need[s] = 1;
            }
            if (!any(need)) break;
            active(need);
            for (int s = 0; s < S; ++s)
                if (need[s]) b.coef(s, std::cos(stp[s]), std::sin(stp[s]));
            k_brotate<T><<<b.nb_el, 256, 0, st>>>(b.d_tab, b.d_esys, b.args);
            OFDFT_LAUNCH_CHECK();
            evaluate(need, BF_NRHO, BF_NV);
            const int r = b.dtheta(BF_NV, BF_NPHI);
            b.sync();
            std::vector<double> En(S, 0.0);
            collect(need, En);
            for (int s = 0; s < S; ++s) {
                if (!need[s]) continue;
                f[s] = En[s];
                gd[s] = 2.0 * b.at(r, s) * dV[s];
                lastE[s] = f[s];
                last_theta[s] = stp[s];
                ++nls[s];
                ++lsit[s];
            }
        }
        std::vector<char> acc(S, 0);
        for (int s = 0; s < S; ++s) {
            if (!run[s]) continue;
            if (ok[s] && natural[s] && theta0[s] > 0.0 && std::isfinite(theta0[s])) last_scale[s] = stp[s] / theta0[s];
            nfev[s] += nls[s];
            if (!ok[s] || nls[s] == 0 || stp[s] != last_theta[s]) {
                conv[s] = 1;  // "Line-Search Failed" (optimization.py:444-448)
                run[s] = 0;
                continue;
            }
            acc[s] = 1;
            accepted_any[s] = 1;
        }
        if (!any(acc)) break;
        // ---- accept
        active(acc);
        b.copy(BF_OLDPHI, BF_PHI);
        b.copy(BF_PHI, BF_NPHI);
        b.copy(BF_V, BF_NV);
        b.square(BF_PHI, BF_RHO);
        for (int s = 0; s < S; ++s)
            if (acc[s]) E[s] = lastE[s];
        b.sum_dev(BF_RHO, SC_D0);
        b.dot_dev(BF_V, BF_RHO, SC_D1);
        b.scalar(OP_MU);
        b.copy(BF_RESPREV, BF_RSD);
        k_bresid_dc<T><<<b.nb_el, 256, 0, st>>>(b.d_tab, b.d_esys, b.args, b.d_sc);
        OFDFT_LAUNCH_CHECK();
        // LBFGS.update (math_utils.py:307-325): at most maxcor+1 pairs
        Pair pr;
        if ((int)lb.size() > o.maxcor) {
            pr = lb.front();
            lb.pop_front();
        } else {
            pr.s = BF_LB0 + pool_i++;
            pr.y = BF_LB0 + pool_i++;
        }
        for (int s = 0; s < S; ++s) b.coef(s, 1.0, -1.0);
        b.lincomb(pr.s, BF_PHI, BF_OLDPHI);
        b.lincomb(pr.y, BF_RSD, BF_RESPREV);
        b.dot_dev(pr.y, pr.s, SC_D0);
        b.scalar(OP_LBRHO, 0, pr.s - BF_LB0);
        const int rres = b.dot(BF_RSD, BF_RSD);
        b.sync();
        lb.push_back(pr);
        for (int s = 0; s < S; ++s) {
            if (!acc[s]) continue;
            Ehist[s].push_back(E[s]);
            dP[s] = b.at(rres, s) * dV[s];
            if (o.verbose)
                fprintf(stderr, "[%d] %-8d%-24.12E%-16.6E%-16.6E%-8d\n", s, it, E[s],
                        Ehist[s][Ehist[s].size() - 1] - Ehist[s][Ehist[s].size() - 2], dP[s], nls[s]);
            // check_converge (optimization.py:527-540)
            const std::vector<double>& H = Ehist[s];
            bool cv = false;
            if ((int)H.size() - 1 >= o.ncheck) {
                cv = true;
                const double ec = econv ? econv[s] : o.econv;
                for (int i = 0; i < o.ncheck; ++i)
                    if (std::fabs(H[H.size() - 2 - i] - E[s]) > ec) cv = false;
            }
            if (cv) {
                conv[s] = 0;
                run[s] = 0;
            }
        }
    }
    for (int s = 0; s < S; ++s)
        if (run[s]) niter[s] = o.maxiter - 1;  // the loop ran out of iterations (conv stays 2), counted as the reference does
    if (o.verbose)
        fprintf(stderr, "batch of %d: %.3f s, %lld evaluations (%.3f s enqueueing), %lld synchronisations (%.3f s "
                "waiting)\n", S,
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count(), b.evals,
                b.enqueue_s, b.syncs, b.wait_s);
    // rho_io <- phi^2, the potential of the last accepted evaluation, results
    std::vector<char> all(S, 1);
    active(all);
    b.square(BF_PHI, BF_RHOIO);
    for (int s = 0; s < S; ++s)
        if (v_out && v_out[s])
            OFDFT_CK(cudaMemcpyAsync(v_out[s], b.h_tab[s].f[BF_V], b.g[s]->real_bytes(), cudaMemcpyDeviceToDevice, st));
    std::vector<char> need_dp(S, 0);
    for (int s = 0; s < S; ++s) need_dp[s] = conv[s] != 0;
    int rdp = -1;
    if (any(need_dp)) {
        active(need_dp);
        rdp = b.dot(BF_RSD, BF_RSD);
    }
    std::vector<double> mu_dev(kBatchMax, 0.0);
    OFDFT_CK(cudaMemcpyAsync(mu_dev.data(), b.d_sc + (size_t)SC_MU * kBatchMax, kBatchMax * sizeof(double),
                             cudaMemcpyDeviceToHost, st));
    b.sync();
    for (int s = 0; s < S; ++s)
        if (accepted_any[s]) mu[s] = mu_dev[s];
    for (int s = 0; s < S; ++s) {
        ofdft_opt_result& r = res[s];
        memset(&r, 0, sizeof(r));
        r.converged = conv[s];
        r.niter = niter[s];
        r.nfev = nfev[s];
        r.energy = E[s];
        r.mu = mu[s];
        r.dP = (conv[s] != 0 && rdp >= 0) ? b.at(rdp, s) * dV[s] : dP[s];
    }
}

}  // namespace

extern "C" {

void ofdft_opt_default(ofdft_opt_options* o) {
    memset(o, 0, sizeof(*o));
    // Optimization defaults (optimization.py:64-78)
    o->method = OFDFT_OPT_CGHS;
    o->maxiter = 200;
    o->maxfun = 50;
    o->maxls = 30;
    o->ncheck = 2;
    o->maxcor = 6;
    o->econv = 1.0e-5;
    o->c1 = 1e-4;
    o->c2 = 0.2;
    o->xtol = 1e-12;
    o->h0 = 1.0;
    o->verbose = 0;
    o->batch_persistent = 0;
    o->pconv = 0.0;
    o->ls_grad = 0;
    o->ls_start = 0;
}

int ofdft_optimize_v(ofdft_eval* e, void* rho, const ofdft_opt_options* o, ofdft_opt_result* r, void* v_out,
                     ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(e && rho && o && r, "ofdft_optimize: null argument");
        OFDFT_REQUIRE(o->method >= OFDFT_OPT_TN && o->method <= OFDFT_OPT_DIIS, "ofdft_optimize: unknown method");
        OFDFT_REQUIRE(o->maxiter >= 1 && o->maxfun >= 1 && o->ncheck >= 1, "ofdft_optimize: bad limits");
        memset(r, 0, sizeof(*r));
        ofdft_grid* g = e_grid(e);
        if (g->prec == OFDFT_F64) optimize_t<double>(e, (double*)rho, *o, *r, (double*)v_out, (cudaStream_t)s);
        else optimize_t<float>(e, (float*)rho, *o, *r, (float*)v_out, (cudaStream_t)s);
    });
}

int ofdft_optimize(ofdft_eval* e, void* rho, const ofdft_opt_options* o, ofdft_opt_result* r, ofdft_stream s) {
    return ofdft_optimize_v(e, rho, o, r, nullptr, s);
}

int ofdft_optimize_batch(int n, ofdft_eval** evs, void** rho, const ofdft_opt_options* o, const double* econv,
                         ofdft_opt_result* r, void** v_out, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(n >= 1 && n <= kBatchMax, "ofdft_optimize_batch: 1..%d systems", kBatchMax);
        OFDFT_REQUIRE(evs && rho && o && r, "ofdft_optimize_batch: null argument");
        OFDFT_REQUIRE(o->maxiter >= 1 && o->maxfun >= 1 && o->ncheck >= 1, "ofdft_optimize_batch: bad limits");
        const int prec = e_grid(evs[0])->prec;
        for (int i = 0; i < n; ++i) {
            OFDFT_REQUIRE(evs[i] && rho[i], "ofdft_optimize_batch: null system %d", i);
            OFDFT_REQUIRE(e_grid(evs[i])->prec == prec, "ofdft_optimize_batch: mixed precisions");
            for (int j = 0; j < i; ++j)
                OFDFT_REQUIRE(e_grid(evs[j]) != e_grid(evs[i]), "ofdft_optimize_batch: systems %d and %d share a grid",
                              j, i);
        }
        if (prec == OFDFT_F64) optimize_batch_t<double>(n, evs, rho, *o, econv, r, v_out, (cudaStream_t)s);
        else optimize_batch_t<float>(n, evs, rho, *o, econv, r, v_out, (cudaStream_t)s);
    });
}

int ofdft_linesearch_grad(ofdft_phi_fn fn, void* ctx, double g0, double stp0, double c2, double amax, int maxiter,
                          double* stp_out, double* f_out, double* g_out, int* nfev) {
    return guard([&] {
        OFDFT_REQUIRE(fn && stp_out && f_out && g_out && nfev, "ofdft_linesearch_grad: null argument");
        bool cb_err = false;
        auto phi = [&](double a, double& f, double& g) {
            if (fn(a, &f, &g, ctx) != 0) cb_err = true;
        };
        double stp = NAN, f = NAN, g = NAN;
        int n = 0;
        bool ok = grad_search(phi, g0, stp0, c2, amax, maxiter, stp, f, g, n);
        OFDFT_REQUIRE(!cb_err, "ofdft_linesearch_grad: callback failed");
        *stp_out = ok ? stp : NAN;
        *f_out = f;
        *g_out = g;
        *nfev = n;
    });
}

int ofdft_linesearch(ofdft_phi_fn fn, void* ctx, double f0, double g0, double stp0, double c1, double c2, double amax,
                     double amin, double xtol, int maxiter, double* stp_out, double* f_out, double* g_out,
                     int* nfev) {
    return guard([&] {
        OFDFT_REQUIRE(fn && stp_out && f_out && g_out && nfev, "ofdft_linesearch: null argument");
        int cb_err = 0;
        auto phi = [&](double a, double& f, double& g) {
            if (fn(a, &f, &g, ctx) != 0) {
                cb_err = 1;
                f = NAN;
                g = NAN;
            }
        };
        double stp, f, g;
        int n = 0;
        bool ok = wolfe1(phi, f0, g0, stp0, c1, c2, amax, amin, xtol, maxiter, stp, f, g, n);
        OFDFT_REQUIRE(!cb_err, "ofdft_linesearch: callback failed");
        *stp_out = ok ? stp : NAN;
        *f_out = f;
        *g_out = g;
        *nfev = n;
    });
}

}  // extern "C"
