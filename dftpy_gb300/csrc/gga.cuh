// GGA kinetic energy functionals (src/dftpy/functional/kedf/gga.py:18-643,
// GGA :1212-1325) and the spectral gradient they share with the vW stress.
//
//   s      = |grad rho| / rho^(4/3) from irfftn(i g rho(G)), rho floored at 1e-16
//   E      = sum C_TF rho^(5/3) F(s) dV
//   V      = 5/3 C_TF rho^(2/3) F - 4/3 tf F' s^2 / rho - div(tf F' grad rho / rho^(8/3))
//            with F' = (1/s) dF/ds, the divergence by irfftn(i g . FFT(...))
//   stress = the reference's GGA stress (:1306-1318)
// One evaluation: 1 R2C, 3 C2R (gradient), 3 R2C and 1 C2R (divergence).
#pragma once
#include "common.cuh"

// included by one translation unit (total.cu)
namespace ofdft {
namespace gga {

// enhancement-factor formulas of the reference's GGA_KEDF_list (gga.py:587-643)
enum GgaFormula {
    GGA_LKT = 0, GGA_LKTVW, GGA_DK, GGA_LLP, GGA_OL, GGA_THAK, GGA_B86A, GGA_B86B, GGA_DK87, GGA_PW86,
    GGA_PW91O, GGA_PW91, GGA_LG94, GGA_P92, GGA_PBE, GGA_P82, GGA_VJKS00, GGA_VT84F, GGA_TFVW, GGA_STV,
    GGA_PBE2M, GGA_PG,
    // MGGA_KEDF_list (gga.py:645-650), F(s, q)
    GGA_GE2, GGA_GE4, GGA_PGSL, GGA_PGSLR, GGA_NFORMULAS
};

struct GgaSpec {
    int formula, np;
    double p[8];
    double remove_vw;  // gga_remove_vw: subtract F = 5/3 pa ss^2 (0: nothing)
    double sigma;      // > 0: gradient smoothed by exp(-G^2 sigma^2/2)
    int meta;          // a Laplacian-level formula (formula >= GGA_GE2)
};

constexpr double kTKF0 = 6.18733545256027186194;      // src/dftpy/constants.py:83
constexpr double kCBRT2 = 1.25992104989487316477;     // src/dftpy/constants.py:84
constexpr double kCTF = 2.87123400018819181594;       // src/dftpy/constants.py:82

// F(s) and F' = (1/s) dF/ds of formula sp.formula at s (the working precision M)
template <typename M>
__device__ inline void gga_formula(const GgaSpec& sp, M s, M& F, M& d) {
    const M p0 = (M)sp.p[0], p1 = (M)sp.p[1], p2 = (M)sp.p[2], p3 = (M)sp.p[3], p4 = (M)sp.p[4], p5 = (M)sp.p[5],
            p6 = (M)sp.p[6];
    const M tk = (M)kTKF0, b = (M)kCBRT2, ctf = (M)kCTF, one = (M)1;
    const M ss = s / tk;  // s_with_tkf0 formulas: in ss, F' rescaled by 1/TKF0^2
    const M s2 = ss * ss;
    bool tkf0 = true;
    switch (sp.formula) {
        case GGA_LKT: {  // LKT_legacy (:547-577)
            if (ss > (M)100) {
                F = (M)(5.0 / 3.0) * s2 * p1;
                d = (M)(10.0 / 3.0) * p1;
            } else if (ss < (M)1e-5) {
                F = one + ((M)(5.0 / 3.0) * p1 - (M)0.5 * p0 * p0) * s2 + (M)(5.0 / 24.0) * (p0 * p0 * p0 * p0) * (s2 * s2);
                d = (M)(10.0 / 3.0) * p1 - p0 * p0 + (M)(5.0 / 6.0) * (p0 * p0 * p0 * p0) * s2 -
                    (M)(61.0 / 120.0) * (p0 * p0 * p0 * p0 * p0 * p0) * (s2 * s2);
            } else {
                const M ch = cosh(p0 * ss);
                F = one / ch + (M)(5.0 / 3.0) * s2 * p1;
                d = (M)(10.0 / 3.0) * p1 - p0 * sinh(p0 * ss) / (ch * ch) / ss;
            }
            break;
        }
        case GGA_LKTVW: {  // LKTmVW (:43-55)
            const M e1 = exp(-p0 * ss), e2 = exp((M)(-2.0) * p0 * ss);
            F = (M)2 * e1 / (one + e2);
            d = -p0 * (one - e2) / (one + e2) * F / ss;
            break;
        }
        case GGA_PW86: {  // (:198-213)
            const M s4 = s2 * s2;
            const M Fa = one + p0 * s2 + p1 * s4 + p2 * (s2 * s4);
            F = pow(Fa, (M)(1.0 / 15.0));
            d = (M)(2.0 / 15.0) * (p0 + 2 * p1 * s2 + 3 * p2 * s4) / pow(Fa, (M)(14.0 / 15.0));
            break;
        }
        case GGA_PW91O: {  // PW910 (:216-239)
            const M s4 = s2 * s2, ex = exp(-p3 * s2);
            const M Fa = (p1 - p2 * ex) * s2 - p5 * s4;
            const M Fb = one + p0 * ss * asinh(p4 * ss) + p5 * s4;
            F = one + Fa / Fb;
            const M Fa_s2 = (p1 - p2 * ex) - p5 * s2;
            d = (M)2 * (p1 + (p3 * s2 - one) * p2 * ex - (M)4 * p5 * s2) / Fb -
                Fa_s2 * ss / (Fb * Fb) * ((p0 * p4 * ss) / (p4 * p4 * s2 + one) + p0 * asinh(p4 * ss) + (M)4 * p5 * s2);
            break;
        }
        case GGA_PW91: {  // PW91 / LC94 (:242-277)
            const M s4 = s2 * s2, ex = exp(-p3 * s2), ash = asinh(p4 * ss);
            const M Fa = one + p0 * ss * ash + (p1 - p2 * ex) * s2;
            const M Fb = one + p0 * ss * ash + p5 * s4;
            F = Fa / Fb;
            const M sq = sqrt(p4 * p4 * s2 + one);
            const M Fa_s = p0 * p4 * ss / sq + p0 * ash + (M)2 * ss * (p1 + (M)2 * p2 * p3 * s2 * ex - (M)2 * p2 * ex);
            d = Fa_s / Fb - Fa / (Fb * Fb) * (p0 * p4 * ss / sq + (p0 * ash + (M)4 * p5 * s2 * ss));
            if (ss > (M)1e-8) d /= ss;
            break;
        }
        case GGA_LG94: {  // (:280-316)
            const M s4 = s2 * s2, s6 = s4 * s2, s8 = s4 * s4, s10 = s4 * s6, s12 = s6 * s6;
            const M Fa = one + p0 * s2 + p1 * s4 + p2 * s6 + p3 * s8 + p4 * s10 + p5 * s12;
            const M Fb = one + (M)1e-8 * s2;
            F = pow(Fa / Fb, p6);
            d = (M)(-2) * p6 * F *
                ((M)1e-8 * Fa - Fb * (p0 + 2 * p1 * s2 + 3 * p2 * s4 + 4 * p3 * s6 + 5 * p4 * s8 + 6 * p5 * s10)) /
                (Fa * Fb);
            break;
        }
        case GGA_P92: {  // (:319-335)
            const M Fa = p0 + p1 * s2 + p2 * (s2 * s2), Fb = p0 + p3 * s2;
            F = Fa / Fb;
            d = ((M)2 * p1 + (M)4 * p2 * s2) / Fb - ((M)2 * p3 * Fa) / (Fb * Fb);
            break;
        }
        case GGA_PBE: {  // (:338-368); the terms present follow the parameter count
            const M Fb = one + p1 / p0 * s2, Fb2 = Fb * Fb;
            F = one + p1 * s2 / Fb;
            d = (M)2 * p1 / Fb2;
            if (sp.np > 2) {
                const M s4 = s2 * s2, Fb3 = Fb2 * Fb;
                F += p2 * s4 / Fb2;
                d += 4 * p2 * s2 / Fb3;
                if (sp.np > 3) {
                    F += p3 * (s4 * s2) / Fb3;
                    d += 6 * p3 * s4 / (Fb3 * Fb);
                }
            }
            break;
        }
        case GGA_P82: {  // (:371-385)
            const M s6 = s2 * s2 * s2, Fb = one + s6;
            F = one + p0 * s2 / Fb;
            d = p0 * ((M)2 / Fb - (M)6 * s6 / (Fb * Fb));
            break;
        }
        case GGA_VJKS00: {  // (:388-404)
            const M s4 = s2 * s2;
            const M Fa = one + p0 * s2 - p2 * (s4 * s2), Fb = one + p1 * s2 + p2 * s4;
            F = Fa / Fb;
            d = ((M)2 * p0 - (M)6 * p2 * s4) / Fb - ((M)2 * p1 + (M)4 * p2 * s2) * Fa / (Fb * Fb);
            break;
        }
        case GGA_VT84F: {  // (:407-433), ss^2 floored at 1e-8
            const M t2 = s2 < (M)1e-8 ? (M)1e-8 : s2, t4 = t2 * t2;
            const M e1 = exp(-p1 * t2), e2 = exp(-p1 * t4), q = one + p0 * t2;
            F = one + (M)(5.0 / 3.0) * t2 + p0 * t2 * e1 / q + (one - e2) * (one / t2 - one);
            d = (M)(10.0 / 3.0) + (M)2 * p0 * e1 * (one - p1 * t2) / q - (M)2 * p0 * t2 * e1 / (q * q) +
                (M)4 * p1 * t2 * (one / t2 - one) * e2 - (M)2 * (one - e2) / t4;
            break;
        }
        case GGA_TFVW: {  // (:436-447)
            F = p0 + (M)(5.0 / 3.0) * p1 * s2;
            d = (M)(10.0 / 3.0) * p1;
            break;
        }
        case GGA_STV: {  // (:450-462)
            const M Fb = p3 + p2 * s2;
            F = p0 + (M)(5.0 / 3.0) * p1 * s2 / Fb;
            d = (M)(5.0 / 3.0) * p1 * ((M)2 / Fb - (M)2 * s2 * p2 / (Fb * Fb));
            break;
        }
        case GGA_PBE2M: {  // (:465-478)
            const M Fb = p0 + p1 * s2;
            F = one + p2 * s2 / Fb;
            d = (M)2 * p2 / (Fb * Fb);
            break;
        }
        case GGA_PG: {  // (:481-490)
            const M Fa = exp(-p0 * s2);
            F = Fa + (M)(5.0 / 3.0) * p1 * s2;
            d = (M)(-2) * p0 * Fa + (M)(10.0 / 3.0) * p1;
            break;
        }
        default:
            tkf0 = false;
            break;
    }
    if (!tkf0) {  // formulas in s itself
        switch (sp.formula) {
            case GGA_DK: {  // (:58-74)
                const M x = s * s / ((M)72 * ctf);
                const M x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
                const M Fa = (M)9 * p5 * x4 + p2 * x3 + p1 * x2 + p0 * x + one;
                const M Fb = p5 * x3 + p4 * x2 + p3 * x + one;
                F = Fa / Fb;
                d = (((M)36 * p5 * x3 + 3 * p2 * x2 + 2 * p1 * x + p0) / Fb -
                     Fa / (Fb * Fb) * ((M)3 * p5 * x2 + (M)2 * p4 * x + p3)) /
                    ((M)36 * ctf);
                break;
            }
            case GGA_LLP: {  // (:77-95)
                const M bs = b * s, bs2 = bs * bs, ash = asinh(bs);
                const M Fa = p0 * bs2, Fb = one + p1 * bs * ash;
                F = one + Fa / Fb;
                d = ((M)2 * p0 / Fb - (p0 * p1 * bs * ash + Fa * p1 / sqrt(one + bs2)) / (Fb * Fb)) * (b * b);
                break;
            }
            case GGA_OL: {  // (:98-112)
                const M q = one + p1 * 4 * s;
                F = one + s * s / (M)72 / ctf + p0 / ctf * s / q;
                d = one / (M)36 / ctf;
                if (s > (M)1e-8) d += p0 / ctf / (q * q) / s;
                break;
            }
            case GGA_THAK: {  // (:115-142)
                const M bs = b * s, bs2 = bs * bs, ash = asinh(bs), c53 = (M)3.1748021039363987;  // 2^(5/3)
                F = one + p0 * bs2 / (one + p1 * bs * ash) - p2 * bs / (one + c53 * bs);
                const M Fb = (one + p1 * bs * ash) * (one + p1 * bs * ash);
                d = (-(p0 * p1 * bs2) / sqrt(one + bs2) + (p0 * p1 * bs * ash) + (M)2 * p0) / Fb;
                if (s > (M)1e-8) d -= p2 / ((one + c53 * bs) * (one + c53 * bs)) / bs;
                d *= b * b;
                break;
            }
            case GGA_B86A: {  // (:145-159)
                const M bs = b * s, bs2 = bs * bs, Fb = one + p1 * bs2;
                F = one + p0 * bs2 / Fb;
                d = 2 * p0 / (Fb * Fb) * (b * b);
                break;
            }
            case GGA_B86B: {  // (:162-176), PowerInt(1 + p1 bs^2, 4, 5)
                const M bs = b * s, bs2 = bs * bs, a = one + p1 * bs2;
                const M Fb = pow(a * a * a * a, (M)(1.0 / 5.0));
                F = one + p0 * bs2 / Fb;
                d = (2 * p0 * (p1 * bs2 + (M)5)) / (5 * a * Fb) * (b * b);
                break;
            }
            case GGA_DK87: {  // (:179-195)
                const M bs = b * s, bs2 = bs * bs;
                const M Fa = p0 * bs2 * (one + p1 * bs), Fb = one + p2 * bs2;
                F = one + Fa / Fb;
                d = p0 * ((M)2 + (M)3 * p1 * bs + p1 * p2 * bs2 * bs) / (Fb * Fb) * (b * b);
                break;
            }
            default:
                F = one;
                d = (M)0;
                break;
        }
    } else {
        d /= tk * tk;
    }
    if (sp.remove_vw != 0.0) {  // gga_remove_vw (:1283-1291): TFVW with [0, pa]
        const M pa = (M)sp.remove_vw;
        F -= (M)(5.0 / 3.0) * pa * s2;
        d -= (M)(10.0 / 3.0) * pa / (tk * tk);
    }
}

// Meta-GGA F(s, q), F' = (1/s) dF/ds and dF/dq (GE2, GE4, PGSL, PGSLr,
// gga.py:492-545), all in ss = s / TKF0 with F' rescaled by 1/TKF0^2, and
// gga_remove_vw as in gga_formula.
template <typename M>
__device__ inline void mgga_formula(const GgaSpec& sp, M s, M q, M& F, M& d, M& dq) {
    const M p0 = (M)sp.p[0], p1 = (M)sp.p[1], p2 = (M)sp.p[2], p3 = (M)sp.p[3], p4 = (M)sp.p[4], p5 = (M)sp.p[5];
    const M tk = (M)kTKF0;
    const M ss = s / tk;
    const M s2 = ss * ss;
    switch (sp.formula) {
        case GGA_GE2:
            F = p0 + p1 * s2 + p2 * q;
            d = (M)2 * p1;
            dq = p2;
            break;
        case GGA_GE4:
            F = (p0 + p1 * s2 + p2 * q) + (p3 * q * q + p4 * q * s2 + p5 * s2 * s2);
            d = (M)2 * p1 + ((M)2 * p4 * q + (M)4 * p5 * s2);
            dq = p2 + ((M)2 * p3 * q + p4 * s2);
            break;
        case GGA_PGSL: {
            const M Fa = exp(-p1 * s2);
            F = Fa + q * q * p0 + (M)(5.0 / 3.0) * p2 * s2;
            d = (M)-2 * p1 * Fa + (M)(10.0 / 3.0) * p2;
            dq = (M)2 * p0 * q;
            break;
        }
        default: {  // GGA_PGSLR: PGSL with the parameters from the third on
            const M Fa = exp(-p3 * s2);
            F = (Fa + q * q * p2 + (M)(5.0 / 3.0) * p4 * s2) + (-p0 * q * s2 + p1 * s2 * s2);
            d = ((M)-2 * p3 * Fa + (M)(10.0 / 3.0) * p4) + ((M)-2 * p0 * q + (M)4 * p1 * s2);
            dq = (M)2 * p2 * q + (-p0 * s2);
            break;
        }
    }
    d /= tk * tk;
    if (sp.remove_vw != 0.0) {
        const M pa = (M)sp.remove_vw;
        F -= (M)(5.0 / 3.0) * pa * s2;
        d -= (M)(10.0 / 3.0) * pa / (tk * tk);
    }
}

// X_d = i g_d FFT(rho) / N, d = 0, 1, 2, as three consecutive planes, and with
// lap != 0 a fourth, -G^2 FFT(rho) / N (DirectField.laplacian, field.py:379-386).
// Under sigma both are smoothed by exp(-G^2 sigma^2/2).  numpy's
// irfftn keeps only the Hermitian part of the k2 = 0 and k2 = n2/2 planes, so
// there a Nyquist frequency index counts as zero; any C2R of X then returns
// numpy's gradient (DirectField.standard_gradient, field.py:267-281).
template <typename T>
__global__ void k_grad_spectra(const typename Cplx<T>::type* __restrict__ rhoG, typename Cplx<T>::type* X, Geo geo,
                               double invN, double sigma, int lap) {
    const double s2 = sigma > 0.0 ? sigma * sigma / 2.0 : 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < geo.Nc; idx += stride) {
        const int k = (int)(idx % geo.n2h);
        const long long t = idx / geo.n2h;
        const int j = (int)(t % geo.n1);
        const int i = (int)(t / geo.n1);
        const bool edge = k == 0 || (geo.n2 % 2 == 0 && k == geo.n2 / 2);
        double f0 = (double)freq_index(i, geo.n0), f1 = (double)freq_index(j, geo.n1), f2 = (double)k;
        if (edge) {
            if (geo.n0 % 2 == 0 && i == geo.n0 / 2) f0 = 0.0;
            if (geo.n1 % 2 == 0 && j == geo.n1 / 2) f1 = 0.0;
            if (geo.n2 % 2 == 0 && k == geo.n2 / 2) f2 = 0.0;
        }
        f0 *= geo.fv[0];
        f1 *= geo.fv[1];
        f2 *= geo.fv[2];
        const double g[3] = {f0 * geo.b[0] + f1 * geo.b[3] + f2 * geo.b[6], f0 * geo.b[1] + f1 * geo.b[4] + f2 * geo.b[7],
                             f0 * geo.b[2] + f1 * geo.b[5] + f2 * geo.b[8]};
        double sc = invN;
        if (s2 > 0.0) sc *= exp(-gsq(geo, idx) * s2);  // field.py:243-248
        const double rr = (double)rhoG[idx].x * sc, ri = (double)rhoG[idx].y * sc;
        for (int d = 0; d < 3; ++d) {
            X[d * geo.Nc + idx].x = (T)(-g[d] * ri);
            X[d * geo.Nc + idx].y = (T)(g[d] * rr);
        }
        if (lap) {
            const double gg = gsq(geo, idx);
            X[3 * geo.Nc + idx].x = (T)(-gg * rr);
            X[3 * geo.Nc + idx].y = (T)(-gg * ri);
        }
    }
}

// Y = i (g . P(G)) / N from the three planes P_d = FFT(p_d), with the same
// Hermitian-part rule on the k2 = 0 and k2 = n2/2 planes (the reference's
// (1j * pot3G).ifft(force_real=True), gga.py:1297-1301)
// With lap != 0, the fourth plane P_q enters as + G^2 exp(-G^2 sigma^2/2) P_q / N:
// minus the Laplacian of p_q (gga.py:1305-1308), as Y is subtracted from pot1.
template <typename T>
__global__ void k_gga_div(const typename Cplx<T>::type* __restrict__ P, typename Cplx<T>::type* Y, Geo geo,
                          double invN, int lap, double sigma) {
    const double s2 = sigma > 0.0 ? sigma * sigma / 2.0 : 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < geo.Nc; idx += stride) {
        const int k = (int)(idx % geo.n2h);
        const long long t = idx / geo.n2h;
        const int j = (int)(t % geo.n1);
        const int i = (int)(t / geo.n1);
        const bool edge = k == 0 || (geo.n2 % 2 == 0 && k == geo.n2 / 2);
        double f0 = (double)freq_index(i, geo.n0), f1 = (double)freq_index(j, geo.n1), f2 = (double)k;
        if (edge) {
            if (geo.n0 % 2 == 0 && i == geo.n0 / 2) f0 = 0.0;
            if (geo.n1 % 2 == 0 && j == geo.n1 / 2) f1 = 0.0;
            if (geo.n2 % 2 == 0 && k == geo.n2 / 2) f2 = 0.0;
        }
        f0 *= geo.fv[0];
        f1 *= geo.fv[1];
        f2 *= geo.fv[2];
        const double g[3] = {f0 * geo.b[0] + f1 * geo.b[3] + f2 * geo.b[6], f0 * geo.b[1] + f1 * geo.b[4] + f2 * geo.b[7],
                             f0 * geo.b[2] + f1 * geo.b[5] + f2 * geo.b[8]};
        double sr = 0.0, si = 0.0;
        for (int d = 0; d < 3; ++d) {
            sr += g[d] * (double)P[d * geo.Nc + idx].x;
            si += g[d] * (double)P[d * geo.Nc + idx].y;
        }
        double yr = -si * invN, yi = sr * invN;
        if (lap) {
            const double gg = gsq(geo, idx);
            double f = gg * invN;
            if (s2 > 0.0) f *= exp(-gg * s2);
            yr += f * (double)P[3 * geo.Nc + idx].x;
            yi += f * (double)P[3 * geo.Nc + idx].y;
        }
        Y[idx].x = (T)yr;
        Y[idx].y = (T)yi;
    }
}

// Pointwise GGA pass over rho and its gradient D (3 planes): energy sum, pot1
// (if pot1 != NULL) and, in place of D, p_d = tf F' d_d rho / rho^(8/3) (if
// want_p).  Partials per block: [0] sum tf F, [1] sum pot1 rho, [2..7] sums of
// w d_i rho d_j rho with w = tf F' / rho^(8/3) (the stress).
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_gga_point(const T* __restrict__ rho, T* D, T* pot1, long long N,
                                                           GgaSpec sp, int want_p, int want_stress, double* partials) {
    using M = T;
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const M ctf = (M)kCTF;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const M r = rho[i];
        const M rm = r < (M)1e-16 ? (M)1e-16 : r;
        const M rho23 = cbrt(rm * rm);  // PowerInt(rhom, 2, 3)
        const M rho53 = rho23 * rm;
        const M tf = ctf * rho53;
        const M rho43 = rho23 * rho23;
        const M rho83 = rho43 * rho43;
        const M dx = D[i], dy = D[N + i], dz = D[2 * N + i];
        M s = sqrt(dx * dx + dy * dy + dz * dz) / rho43;
        if (s < (M)1e-16) s = (M)1e-16;
        M F, dF, dq = (M)0, q = (M)0;
        if (sp.meta) {
            q = D[3 * N + i] / (M)(kTKF0 * kTKF0) / rho53;  // gga.py:1254-1257
            mgga_formula(sp, s, q, F, dF, dq);
        } else {
            gga_formula(sp, s, F, dF);
        }
        acc[0] += (double)(tf * F);
        if (pot1 || want_stress) {
            M p1 = (M)(5.0 / 3.0) * ctf * rho23 * F + (M)(-4.0 / 3.0) * tf * dF * s * s / rm;
            if (sp.meta) {  // tf dF/dq dq0, and p_q = tf dF/dq dq2 for the Laplacian (gga.py:1305-1308)
                p1 += tf * dq * ((M)(-5.0 / 3.0) * q / rm);
                if (want_p) D[3 * N + i] = tf * dq * ((M)(1.0 / (kTKF0 * kTKF0)) / rho53);
            }
            if (pot1) pot1[i] = p1;
            const M w = tf * dF / rho83;
            if (want_stress) {
                acc[1] += (double)p1 * (double)r;
                acc[2] += (double)(w * dx * dx);
                acc[3] += (double)(w * dx * dy);
                acc[4] += (double)(w * dx * dz);
                acc[5] += (double)(w * dy * dy);
                acc[6] += (double)(w * dy * dz);
                acc[7] += (double)(w * dz * dz);
            }
            if (want_p) {
                D[i] = w * dx;
                D[N + i] = w * dy;
                D[2 * N + i] = w * dz;
            }
        }
    }
    block_sum_store<8>(acc, partials);
}

// HC k_F field (hc.py:88-138): rho clamped at 1e-30, s = |D| / rho^(4/3) from
// the gradient D of the clamped density (not floored), F and F' of the
// enhancement factor, k_F = F (3 pi^2 rho)^(1/3); for the potential
// c1 = k_F,std (F - 4 F' s^2) / (3 rho) and c2 = k_F,std F' / rho^(8/3)
// (hc.py:312-313).  Partials: [0] min k_F, [1] max k_F.
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_hc_point(const T* __restrict__ rho, const T* __restrict__ D, T* kf,
                                                          T* c1, T* c2, long long N, GgaSpec sp, double* partials) {
    using M = T;
    M kmin = (M)INFINITY, kmax = -(M)INFINITY;
    const M threepi2 = (M)(3.0 * M_PI * M_PI);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const M r = rho[i];
        const M rc = r < (M)1e-30 ? (M)1e-30 : r;
        const M rho43 = pow(rc, (M)(4.0 / 3.0));
        const M rho83 = rho43 * rho43;
        const M dx = D[i], dy = D[N + i], dz = D[2 * N + i];
        const M s = sqrt(dx * dx + dy * dy + dz * dz) / rho43;
        M F, dF;
        gga_formula(sp, s, F, dF);
        const M kstd = cbrt(threepi2 * rc);
        const M k = F * kstd;
        kf[i] = k;
        if (c1) {
            c1[i] = kstd / ((M)3 * rc) * (F - (M)4 * dF * s * s);
            c2[i] = kstd * dF / rho83;
        }
        kmin = k < kmin ? k : kmin;
        kmax = k > kmax ? k : kmax;
    }
    double acc[2] = {(double)kmin, (double)kmax};
    const int kinds[2] = {1, 2};
    block_reduce_store<2>(acc, kinds, partials);
}

// rho clamped at 1e-30 (hc.py:88-90)
template <typename T>
__global__ void k_hc_clamp(const T* __restrict__ rho, T* out, long long N) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const T r = rho[i];
        out[i] = r < (T)1e-30 ? (T)1e-30 : r;
    }
}

// p_d = d_d rho c2 rho^alpha pot3, in place of the gradient planes (hc.py:313-318)
template <typename T>
__global__ void k_hc_p(T* D, const T* __restrict__ c2, const T* __restrict__ pa, const T* __restrict__ pot3,
                       long long N) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const T w = c2[i] * (pa[i] * pot3[i]);
        D[i] *= w;
        D[N + i] *= w;
        D[2 * N + i] *= w;
    }
}

// V (+)= pot1 - q
template <typename T>
__global__ void k_gga_combine(T* V, const T* __restrict__ pot1, const T* __restrict__ q, long long N, int accumulate) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += stride) {
        const T v = pot1[i] - q[i];
        V[i] = accumulate ? V[i] + v : v;
    }
}

// Enqueue one GGA evaluation on st: 8 partial sums reduced into out_dev[0..7]
// (energy sum, stress sums; the caller scales by dV), V (+)= the GGA potential
// when V != NULL.
template <typename T>
void gga_enqueue(ofdft_grid* g, Scratch& sc, const GgaSpec& sp, const T* rho, T* V, bool accumulate,
                 bool want_stress, double* out_dev, cudaStream_t st) {
    using C = typename Cplx<T>::type;
    const size_t rb = g->real_bytes(), cb = g->cplx_bytes();
    const int gblk = blocks_for(g->Nc, 256, g->sms * 16);
    const int rblk = blocks_for(g->N, 256, g->sms * 16);
    C* rhoG = (C*)sc.get("gga_rhoG", cb);
    const int np = sp.meta ? 4 : 3;  // gradient planes, and the Laplacian for a meta-GGA
    C* X = (C*)sc.get("gga_X", np * cb);
    T* D = (T*)sc.get("gga_D", np * rb);
    T* pot1 = V ? (T*)sc.get("gga_pot1", rb) : nullptr;
    g->exec_r2c(rho, rhoG, 1, st);
    k_grad_spectra<T><<<gblk, 256, 0, st>>>(rhoG, X, g->geo, 1.0 / (double)g->N, sp.sigma, sp.meta);
    OFDFT_LAUNCH_CHECK();
    g->exec_c2r(X, D, np, st);
    k_gga_point<T><<<g->red_blocks, RED_THREADS, 0, st>>>(rho, D, pot1, g->N, sp, V ? 1 : 0, want_stress ? 1 : 0,
                                                          g->d_partials);
    OFDFT_LAUNCH_CHECK();
    reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 8, 0ull, out_dev);
    OFDFT_LAUNCH_CHECK();
    if (!V) return;
    g->exec_r2c(D, X, np, st);
    k_gga_div<T><<<gblk, 256, 0, st>>>(X, rhoG, g->geo, 1.0 / (double)g->N, sp.meta, sp.sigma);
    OFDFT_LAUNCH_CHECK();
    T* q = D;  // the first gradient plane is free again
    g->exec_c2r(rhoG, q, 1, st);
    k_gga_combine<T><<<rblk, 256, 0, st>>>(V, pot1, q, g->N, accumulate ? 1 : 0);
    OFDFT_LAUNCH_CHECK();
}

}  // namespace gga
}  // namespace ofdft
