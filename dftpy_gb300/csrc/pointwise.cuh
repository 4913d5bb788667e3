// Pointwise physics shared by the single-system evaluator and the persistent
// batched evaluator: the TF and LDA constants, Slater + PZ81 exchange-
// correlation at one point (xc/semilocal_xc.py:283-319), working-precision
// math and the per-thread compensated running sum.
#pragma once
#include "common.cuh"

#include <cmath>

namespace {

constexpr double kZERO = 1e-30;  // src/dftpy/constants.py:85

struct Consts {
    double cTF_E, cTF_V;             // TF energy / potential prefactors
    double lda_rs, lda_ex, lda_vx;   // cbrt(3/(4 pi)), -3/4 cbrt(3/pi), cbrt(-3/pi)
    double threepi2;                 // 3 pi^2
    double cTF_wt;                   // 0.3 (3 pi^2)^(2/3)
};

Consts make_consts() {
    Consts c;
    const double pi = M_PI;
    c.cTF_E = (3.0 / 10.0) * std::pow(3.0 * pi * pi, 2.0 / 3.0);
    c.cTF_V = (3.0 / 10.0) * (5.0 / 3.0) * std::pow(3.0 * pi * pi, 2.0 / 3.0);
    c.lda_rs = std::cbrt(3.0 / (4.0 * pi));
    c.lda_ex = -3.0 / 4.0 * std::cbrt(3.0 / pi);
    c.lda_vx = std::cbrt(-3.0 / pi);
    c.threepi2 = 3.0 * pi * pi;
    c.cTF_wt = 0.3 * std::pow(3.0 * pi * pi, 2.0 / 3.0);
    return c;
}

// PZ81 correlation parameters, unpolarised (xc/semilocal_xc.py:287-293)
__constant__ double cPZ[7] = {0.0311, -0.048, 0.0020, -0.0116, -0.1423, 1.0529, 0.3334};
__constant__ float cPZf[7] = {0.0311f, -0.048f, 0.0020f, -0.0116f, -0.1423f, 1.0529f, 0.3334f};

// Working-precision math: float64 for the FP64 path, float32 for FP32-mixed
// (GB300 runs float64 at a small fraction of the float32 rate).
__device__ inline double mcbrt(double x) { return cbrt(x); }
__device__ inline float mcbrt(float x) { return cbrtf(x); }
__device__ inline double mlog(double x) { return log(x); }
__device__ inline float mlog(float x) { return logf(x); }
__device__ inline double msqrt(double x) { return sqrt(x); }
__device__ inline float msqrt(float x) { return sqrtf(x); }
__device__ inline double mpow(double x, double y) { return pow(x, y); }
__device__ inline float mpow(float x, float y) { return powf(x, y); }
__device__ inline double mexp(double x) { return exp(x); }
__device__ inline float mexp(float x) { return expf(x); }
template <typename M>
__device__ inline M pz(int k) {
    return sizeof(M) == 8 ? (M)cPZ[k] : (M)cPZf[k];
}

// Constants of the built-in LDA in the working precision M
template <typename M>
struct LdaC {
    M rs, ex, vx, tiny;
    M P[7];
    __device__ explicit LdaC(const Consts& k)
        : rs((M)k.lda_rs), ex((M)k.lda_ex), vx((M)k.lda_vx), tiny((M)1e-30) {
        for (int i = 0; i < 7; ++i) P[i] = pz<M>(i);
    }
};

// Slater exchange + PZ81 correlation energy per electron ex and potential vx
// at density r (xc/semilocal_xc.py:283-319)
template <typename M>
__device__ __forceinline__ void lda_point(M r, const LdaC<M>& c, M& ex, M& vx) {
    M rc = mcbrt(r);
    if (rc < c.tiny) rc = c.tiny;
    const M Rs = c.rs / rc;
    const M* P = c.P;
    if (Rs < (M)1) {
        const M lr = mlog(Rs);
        ex = c.ex * rc + (P[0] * lr + P[1] + P[2] * Rs * lr + P[3] * Rs);
        vx = c.vx * rc +
             (lr * (P[0] + (M)(2.0 / 3) * P[2] * Rs) + P[1] - (M)(1.0 / 3) * P[0] + (M)(1.0 / 3) * (2 * P[3] - P[2]) * Rs);
    } else {
        const M sRs = msqrt(Rs);
        const M den = (M)1 + P[5] * sRs + P[6] * Rs;
        ex = c.ex * rc + P[4] / den;
        vx = c.vx * rc + (P[4] + ((M)(7.0 / 6.0) * P[4] * P[5]) * sRs + ((M)(4.0 / 3.0) * P[4] * P[6] * Rs)) / (den * den);
    }
}

// Per-thread running sum of a field reduction: float64 in the FP64 path; in the
// FP32 path a float32 Kahan-compensated sum over the thread's points (GB300
// runs float64 at a small fraction of the float32 rate), handed to the float64
// block and grid reductions at the end.
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
    __device__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ double get() const { return (double)s - (double)c; }
};

// Inverse Lindhard function F(eta; lbda, mu) with the reference's four
// branches (kedf/kernel.py:14-136)
__device__ inline double lindhard_dev(double eta, double lbda, double mu) {
    const double tol = 1e-10, tol2 = tol / 10;
    double out = eta;
    if (eta > tol2 && fabs(eta - 1.0) > tol2)
        out = 1.0 / (0.5 + 0.25 * (1.0 - eta * eta) * log((1.0 + eta) / fabs(1.0 - eta)) / eta) - 3.0 * mu * eta * eta -
              lbda;
    if (eta < tol) out = 1.0 - lbda + eta * eta * (1.0 / 3.0 - 3.0 * mu);
    if (fabs(eta - 1.0) < tol) out = 2.0 - lbda - 3.0 * mu + 20.0 * (eta - 1.0);
    if (eta > 3.65) {
        const double c[15] = {-0.13714285714285712, -6.39999999999999875e-2, -3.77825602968460128e-2,
                              -2.51824061652633074e-2, -1.80879839616166146e-2, -1.36715733124818332e-2,
                              -1.07236045520990083e-2, -8.65192783339199453e-3, -7.1372762502456763e-3,
                              -5.9945117538835746e-3, -5.10997527675418131e-3, -4.41060829979912465e-3,
                              -3.84763737842981233e-3, -3.38745061493813488e-3, -3.00624946457977689e-3};
        double inv2 = 1.0 / (eta * eta);
        double acc = c[14] * inv2;
#pragma unroll
        for (int k = 13; k >= 0; --k) acc = inv2 * (c[k] + acc);
        out = 3.0 * (1.0 - mu) * eta * eta - lbda - 0.6 + acc;
    }
    return out;
}

}  // namespace
