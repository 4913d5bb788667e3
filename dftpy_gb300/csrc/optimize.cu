// Density optimisation on phi = sqrt(rho) (Optimization.optimize_rho,
// src/dftpy/optimization/optimization.py:283-525) with the line search of
// scipy's line_search_wolfe1 (math_utils.py:37-52): the MINPACK-2 routine
// dcsrch/dcstep of More and Thuente (ACM TOMS 20, 1994), restated here.
// All field work stays on the device; only scalars (energies, dot products,
// line-search state) live on the host.
#include "common.cuh"

#include <algorithm>
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

template <typename T>
__global__ void k_lincomb(long long n, T* out, double a0, const T* x0, double a1, const T* x1, double a2,
                          const T* x2) {
    const T b0 = (T)a0, b1 = (T)a1, b2 = (T)a2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        T v = b0 * x0[i];
        if (x1) v += b1 * x1[i];
        if (x2) v += b2 * x2[i];
        out[i] = v;
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
        out[i] = v * v;
    }
}

// newphi = phi cos + p sin, rho = newphi^2
template <typename T>
__global__ void k_rotate(long long n, const T* phi, const T* p, double c, double s, T* newphi, T* rho) {
    const T cw = (T)c, sw = (T)s;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const T v = phi[i] * cw + p[i] * sw;
        newphi[i] = v;
        rho[i] = v * v;
    }
}

// out = (V - mu) phi
template <typename T>
__global__ void k_resid(long long n, const T* V, double mu, const T* phi, T* out) {
    const T m = (T)mu;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (V[i] - m) * phi[i];
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
        sum.add(V[i] * nphi[i] * (p[i] * cw - phi[i] * sw));
    double acc[1] = {sum.get()};
    block_sum_store<1>(acc, partials);
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_dot2(long long n, const T* a, const T* b, double* partials) {
    RunSum<T> sum;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        sum.add(a[i] * b[i]);
    double acc[1] = {sum.get()};
    block_sum_store<1>(acc, partials);
}

}  // namespace

// grid of an evaluator (the evaluator struct lives in total.cu)
ofdft_grid* e_grid(ofdft_eval* e);

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
    for (it = 1; it < o.maxiter; ++it) {
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
        } else {
            // get_direction_CG, CG-HS (math_utils.py:328-361)
            if (have_res_prev && have_dir_prev) {
                T* dr = op.buf("cg_dr");
                op.lincomb(dr, 1.0, rsd, -1.0, res_prev);
                double beta = op.dot(rsd, dr) / op.dot(dir_prev, dr);
                op.lincomb(p, -1.0, rsd, beta, dir_prev);
            } else {
                op.lincomb(p, -1.0, rsd);
            }
        }
        double theta0 = op.orth_norm(p, phi);
        (void)theta0;
        if (op.dtheta(V, phi, p, phi, 1.0, 0.0) * 2.0 > 0) {
            // uphill: steepest descent (optimization.py:373-380)
            op.lincomb(p, -1.0, rsd);
            op.orth_norm(p, phi);
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
        bool ok = wolfe1(phi_fn, E, g0, 1.0, o.c1, o.c2, M_PI, 0.0, o.xtol, 100, stp, fnew, gnew, nls);
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
    res.niter = it;
    res.nfev = nfev;
    res.energy = E;
    res.mu = mu;
    if (converged != 0) res.dP = op.dot(rsd, rsd) * dV;
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
}

int ofdft_optimize_v(ofdft_eval* e, void* rho, const ofdft_opt_options* o, ofdft_opt_result* r, void* v_out,
                     ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(e && rho && o && r, "ofdft_optimize: null argument");
        OFDFT_REQUIRE(o->method >= 0 && o->method <= 2, "ofdft_optimize: unknown method");
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
