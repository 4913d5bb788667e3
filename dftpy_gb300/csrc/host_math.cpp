// Host-side numerics: not-a-knot cubic splines, inverse Lindhard function,
// k_F node rules, cardinal B-splines, inverse erfc.
#include "host_math.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <stdexcept>

namespace ofdft {

void CubicSpline::fit(const std::vector<double>& xs, const std::vector<double>& ys) {
    const int n = (int)xs.size();
    if (n < 4 || (int)ys.size() != n) throw std::invalid_argument("CubicSpline needs >= 4 points");
    x = xs;
    std::vector<double> h(n - 1), d(n - 1);
    for (int i = 0; i < n - 1; ++i) {
        h[i] = xs[i + 1] - xs[i];
        if (!(h[i] > 0)) throw std::invalid_argument("CubicSpline: x not increasing");
        d[i] = (ys[i + 1] - ys[i]) / h[i];
    }
    // Second derivatives M_i.  Interior rows i = 1..n-2:
    //   h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1} = 6 (d_i - d_{i-1}).
    // Not-a-knot: the third derivative is continuous at x_1 and x_{n-2}, i.e.
    //   M_0 = M_1 (1 + h0/h1) - M_2 h0/h1 and the mirror relation at the end;
    // substituting them leaves a tridiagonal system in M_1..M_{n-2}.
    const int m = n - 2;
    std::vector<double> lo(m), di(m), up(m), rhs(m);
    for (int r = 0; r < m; ++r) {
        int i = r + 1;
        lo[r] = h[i - 1];
        di[r] = 2.0 * (h[i - 1] + h[i]);
        up[r] = h[i];
        rhs[r] = 6.0 * (d[i] - d[i - 1]);
    }
    {
        double a = h[0] / h[1];
        di[0] += lo[0] * (1.0 + a);
        up[0] -= lo[0] * a;
        lo[0] = 0.0;
        double b = h[n - 2] / h[n - 3];
        di[m - 1] += up[m - 1] * (1.0 + b);
        lo[m - 1] -= up[m - 1] * b;
        up[m - 1] = 0.0;
    }
    std::vector<double> M(n);
    if (m == 1) {
        M[1] = rhs[0] / di[0];
    } else {
        // Thomas algorithm
        for (int r = 1; r < m; ++r) {
            double w = lo[r] / di[r - 1];
            di[r] -= w * up[r - 1];
            rhs[r] -= w * rhs[r - 1];
        }
        M[m] = rhs[m - 1] / di[m - 1];
        for (int r = m - 2; r >= 0; --r) M[r + 1] = (rhs[r] - up[r] * M[r + 2]) / di[r];
    }
    {
        double a = h[0] / h[1];
        M[0] = M[1] * (1.0 + a) - M[2] * a;
        double b = h[n - 2] / h[n - 3];
        M[n - 1] = M[n - 2] * (1.0 + b) - M[n - 3] * b;
    }
    c.assign(4 * (n - 1), 0.0);
    for (int i = 0; i < n - 1; ++i) {
        c[4 * i + 0] = ys[i];
        c[4 * i + 1] = d[i] - h[i] * (2.0 * M[i] + M[i + 1]) / 6.0;
        c[4 * i + 2] = 0.5 * M[i];
        c[4 * i + 3] = (M[i + 1] - M[i]) / (6.0 * h[i]);
    }
}

std::vector<double> CubicSpline::adjoint(const std::vector<double>& gc) const {
    const int n = (int)x.size();
    std::vector<double> h(n - 1);
    for (int i = 0; i < n - 1; ++i) h[i] = x[i + 1] - x[i];
    const int m = n - 2;
    // the (modified) tridiagonal system of fit()
    std::vector<double> lo(m), di(m), up(m);
    for (int r = 0; r < m; ++r) {
        int i = r + 1;
        lo[r] = h[i - 1];
        di[r] = 2.0 * (h[i - 1] + h[i]);
        up[r] = h[i];
    }
    const double a = h[0] / h[1], b = h[n - 2] / h[n - 3];
    di[0] += lo[0] * (1.0 + a);
    up[0] -= lo[0] * a;
    lo[0] = 0.0;
    di[m - 1] += up[m - 1] * (1.0 + b);
    lo[m - 1] -= up[m - 1] * b;
    up[m - 1] = 0.0;
    std::vector<double> gy(n, 0.0), gd(n - 1, 0.0), gM(n, 0.0);
    // coefficients -> (y, d, M)
    for (int i = 0; i < n - 1; ++i) {
        const double g0 = gc[4 * i], g1 = gc[4 * i + 1], g2 = gc[4 * i + 2], g3 = gc[4 * i + 3];
        gy[i] += g0;
        gd[i] += g1;
        gM[i] += -h[i] * 2.0 / 6.0 * g1 + 0.5 * g2 - g3 / (6.0 * h[i]);
        gM[i + 1] += -h[i] / 6.0 * g1 + g3 / (6.0 * h[i]);
    }
    // not-a-knot end relations M_0(M_1, M_2), M_{n-1}(M_{n-2}, M_{n-3})
    gM[1] += gM[0] * (1.0 + a);
    gM[2] -= gM[0] * a;
    gM[n - 2] += gM[n - 1] * (1.0 + b);
    gM[n - 3] -= gM[n - 1] * b;
    // interior solve: rhs adjoint = T^-T gM_interior (Thomas on the transpose)
    std::vector<double> tl(m), td(m), tu(m), g(m);
    for (int r = 0; r < m; ++r) {
        td[r] = di[r];
        tl[r] = r > 0 ? up[r - 1] : 0.0;
        tu[r] = r < m - 1 ? lo[r + 1] : 0.0;
        g[r] = gM[r + 1];
    }
    if (m == 1) {
        g[0] /= td[0];
    } else {
        for (int r = 1; r < m; ++r) {
            double w = tl[r] / td[r - 1];
            td[r] -= w * tu[r - 1];
            g[r] -= w * g[r - 1];
        }
        g[m - 1] /= td[m - 1];
        for (int r = m - 2; r >= 0; --r) g[r] = (g[r] - tu[r] * g[r + 1]) / td[r];
    }
    // rhs_r = 6 (d_{r+1} - d_r)
    for (int r = 0; r < m; ++r) {
        gd[r + 1] += 6.0 * g[r];
        gd[r] -= 6.0 * g[r];
    }
    // d_i = (y_{i+1} - y_i) / h_i
    for (int i = 0; i < n - 1; ++i) {
        gy[i + 1] += gd[i] / h[i];
        gy[i] -= gd[i] / h[i];
    }
    return gy;
}

int CubicSpline::interval(double xv) const {
    const int n = (int)x.size();
    if (xv <= x[0]) return 0;
    if (xv >= x[n - 1]) return n - 2;
    int i = (int)(std::upper_bound(x.begin(), x.end(), xv) - x.begin()) - 1;
    return std::min(std::max(i, 0), n - 2);
}

double CubicSpline::eval(double xv) const {
    int i = interval(xv);
    double u = xv - x[i];
    const double* q = &c[4 * i];
    return q[0] + u * (q[1] + u * (q[2] + u * q[3]));
}

double CubicSpline::deriv(double xv) const {
    int i = interval(xv);
    double u = xv - x[i];
    const double* q = &c[4 * i];
    return q[1] + u * (2.0 * q[2] + u * 3.0 * q[3]);
}

static const double kLarge[15] = {-0.13714285714285712, -6.39999999999999875e-2, -3.77825602968460128e-2,
                                  -2.51824061652633074e-2, -1.80879839616166146e-2, -1.36715733124818332e-2,
                                  -1.07236045520990083e-2, -8.65192783339199453e-3, -7.1372762502456763e-3,
                                  -5.9945117538835746e-3, -5.10997527675418131e-3, -4.41060829979912465e-3,
                                  -3.84763737842981233e-3, -3.38745061493813488e-3, -3.00624946457977689e-3};

double lindhard(double eta, double lbda, double mu) {
    const double tol = 1e-10, tol2 = tol / 10;
    // later branches override earlier ones, as in the reference
    double out = eta;
    if (eta > tol2 && std::fabs(eta - 1.0) > tol2)
        out = 1.0 / (0.5 + 0.25 * (1.0 - eta * eta) * std::log((1.0 + eta) / std::fabs(1.0 - eta)) / eta) -
              3.0 * mu * eta * eta - lbda;
    if (eta < tol) out = 1.0 - lbda + eta * eta * (1.0 / 3.0 - 3.0 * mu);
    if (std::fabs(eta - 1.0) < tol) out = 2.0 - lbda - 3.0 * mu + 20.0 * (eta - 1.0);
    if (eta > 3.65) {
        double inv2 = 1.0 / (eta * eta);
        double acc = kLarge[14] * inv2;
        for (int k = 13; k >= 0; --k) acc = inv2 * (kLarge[k] + acc);
        out = 3.0 * (1.0 - mu) * eta * eta - lbda - 0.6 + acc;
    }
    return out;
}

std::vector<double> mgp_kernel_table(const std::vector<double>& eta, int maxpoints, int sym) {
    const int n = (int)eta.size();
    if (n < 4) throw std::invalid_argument("MGP table needs >= 4 points");
    // F(eta; 1, 1) as a cubic spline on numpy's logspace(log10(eta[1]/10), log10(eta[-1]+2), n)
    const double a = std::log10(eta[1] / 10.0), b = std::log10(eta[n - 1] + 2.0);
    const double step = (b - a) / (double)(n - 1);
    std::vector<double> gp(n), f(n);
    for (int i = 0; i < n; ++i) gp[i] = std::pow(10.0, i == n - 1 ? b : a + (double)i * step);
    for (int i = 0; i < n; ++i) f[i] = lindhard(gp[i], 1.0, 1.0);
    CubicSpline S;
    S.fit(gp, f);
    // sum over t = i/maxpoints of F(eta t^-1/3) / t^(1/6) (t^(-2/3) geometric), F
    // extended by its end values outside the grid (splev ext=3); eta t^-1/3 grows
    // with eta, so each pass walks the intervals forward
    const double dt = 1.0 / (double)maxpoints;
    std::vector<double> ker(n, 0.0);
    for (int i = 1; i <= maxpoints; ++i) {
        const double t = (double)i * dt;
        const double ct = std::cbrt(t);
        const double t16 = sym == 2 ? std::pow(t, -2.0 / 3.0) : std::pow(t, 1.0 / 6.0);
        int l = 0;
        for (int j = 0; j < n; ++j) {
            double x = eta[j] / ct;
            x = x < gp[0] ? gp[0] : (x > gp[n - 1] ? gp[n - 1] : x);
            while (l < n - 2 && x >= gp[l + 1]) ++l;
            const double u = x - gp[l];
            const double* c = S.c.data() + 4 * (size_t)l;
            ker[j] += (c[0] + u * (c[1] + u * (c[2] + u * c[3]))) / t16;
        }
    }
    const double cTF = 0.3 * std::pow(3.0 * M_PI * M_PI, 2.0 / 3.0);
    const double coe = 4.0 / 5.0 * cTF * 5.0 / 6.0 * dt;
    const double wt_factor = 4.0 / 5.0 * cTF;
    for (int j = 0; j < n; ++j) {
        if (sym == 1) ker[j] = 0.5 * (ker[j] * coe + lindhard(eta[j], 1.0, 1.0) * wt_factor);
        else if (sym == 2) ker[j] *= 2.0 * coe;
        else ker[j] *= coe;
    }
    return ker;
}

void guess_kf_bound(double kf_l, double kf_r, bool fixed_min, double kfmin_in, bool fixed_max, double kfmax_in,
                    bool& set_min, double& st_min, bool& set_max, double& st_max, double& out_min, double& out_max) {
    if (fixed_min && fixed_max) {
        out_min = kfmin_in;
        out_max = kfmax_in;
        return;
    }
    bool have_min = fixed_min, have_max = fixed_max;
    double kfmin = kfmin_in, kfmax = kfmax_in;
    double pmin, pmax;
    if (!set_min) {
        pmin = 10.0;
        if (!have_min) {
            kfmin = kf_l;
            have_min = true;
        }
    } else {
        pmin = st_min;
    }
    if (!set_max) {
        pmax = 1.0;
        if (!have_max) {
            kfmax = kf_r;
            have_max = true;
        }
    } else {
        pmax = st_max;
    }
    if (!have_min || kfmin > pmin) kfmin = pmin;
    if (!have_max || kfmax < pmax) kfmax = pmax;
    if (kfmin > kf_l) {
        static const double kfl[10] = {1e-5, 1e-4, 5e-3, 1e-3, 5e-3, 1e-2, 5e-2, 0.1, 0.5, 1.0};
        double ratio = kf_l / kfmin;
        for (int i = 9; i > 0; --i) {
            if (ratio > kfl[i]) {
                kfmin *= kfl[i];
                break;
            }
        }
    }
    if (kfmin < 1e-3) kfmin = 1e-3;
    if (kfmax < kf_r) {
        double dk = kf_r - kfmax;
        kfmax += (std::nearbyint(dk / 0.5) + 1.0) * 0.5;
    }
    set_min = set_max = true;
    st_min = kfmin;
    st_max = kfmax;
    out_min = kfmin;
    out_max = kfmax;
}

std::vector<double> hc_kf_nodes(double kf_l, double kf_r, bool fixed_min, double kfmin_in, bool fixed_max,
                                double kfmax_in, bool& set_min, double& st_min, bool& set_max, double& st_max,
                                double ratio, int nsp, double delta) {
    const double kf0 = 1.0;
    double kfmin = kfmin_in, kfmax = kfmax_in;
    if (!fixed_min) {
        kfmin = std::max(kf_l, 1e-3);
        const int n = (int)std::floor(std::log(kfmin / kf0) / std::log(ratio)) - 1;
        kfmin = kf0 * std::pow(ratio, (double)n);
    }
    if (!fixed_max) {
        kfmax = std::min(kf_r, 100.0);
        const int n = (int)std::ceil(std::log(kfmax / kf0) / std::log(ratio)) + 1;
        kfmax = kf0 * std::pow(ratio, (double)n);
    }
    if (set_min && kfmin > st_min && (kfmin - st_min) < 0.2) kfmin = st_min;
    if (set_max && kfmax < st_max && (st_max - kfmax) < 1) kfmax = st_max;
    std::vector<double> k;
    if (nsp > 0) {
        if (kfmax - kfmin < 1e-3) {
            k = {kfmin, kfmax};
        } else {
            const double step = (kfmax - kfmin) / (double)(nsp - 1);
            k.resize(nsp);
            for (int i = 0; i < nsp; ++i) k[i] = kfmin + step * (double)i;
        }
    } else if (delta > 0) {
        const int n = (int)std::ceil((kfmax - kfmin) / delta) + 1;
        k.resize(n);
        if (n == 1) {
            k[0] = kfmin;
        } else {
            const double step = (kfmax - kfmin) / (double)(n - 1);
            for (int i = 0; i < n; ++i) k[i] = (double)i * step + kfmin;
            k[n - 1] = kfmax;
        }
    } else {
        const int n = (int)(std::log(kfmax / kfmin) / std::log(ratio)) + 1;
        k.resize(n);
        for (int i = 0; i < n; ++i) k[i] = kfmin * std::pow(ratio, (double)i);
    }
    k.front() -= 1e-16;  // savetol
    k.back() += 1e-16;
    set_min = set_max = true;
    st_min = kfmin;
    st_max = kfmax;
    return k;
}

std::vector<double> kf_nodes(double kfMin, double kfMax, int nsp, double delta, double ratio) {
    std::vector<double> k;
    if (nsp > 0) {
        if (kfMax - kfMin < 1e-3) {
            k = {kfMin, kfMax};
        } else {
            double step = (kfMax - kfMin) / (double)(nsp - 1);
            k.resize(nsp);
            for (int i = 0; i < nsp; ++i) k[i] = kfMin + step * (double)i;
        }
    } else if (delta > 0) {
        int n = (int)std::ceil((kfMax - kfMin) / delta) + 1;
        // numpy linspace: step = (stop-start)/(n-1); y = arange*step + start; y[-1] = stop
        k.resize(n);
        if (n == 1) {
            k[0] = kfMin;
        } else {
            double step = (kfMax - kfMin) / (double)(n - 1);
            for (int i = 0; i < n; ++i) k[i] = (double)i * step + kfMin;
            k[n - 1] = kfMax;
        }
    } else {
        int n = (int)std::ceil(std::log(kfMax / kfMin) / std::log(ratio)) + 1;
        k.resize(n);
        for (int i = 0; i < n; ++i) k[i] = kfMin * std::pow(ratio, (double)i);
    }
    k.front() -= 1e-16;
    k.back() += 1e-16;
    return k;
}

void bspline_mn(double x, int order, int order_full, double* Mn) {
    for (int i = 0; i <= order_full; ++i) Mn[i] = 0.0;
    Mn[1] = x;
    Mn[2] = 1.0 - x;
    for (int i = 3; i <= order; ++i) {
        for (int j = 0; j < i; ++j) {
            int n = i - j;
            Mn[n] = (x + n - 1) * Mn[n] + (j + 1 - x) * Mn[n - 1];
            Mn[n] /= (double)(i - 1);
        }
    }
}

void bspline_bm(int n, int nG, int order, std::vector<double>& re, std::vector<double>& im) {
    std::vector<double> Mn(order + 1);
    bspline_mn(1.0, order, order, Mn.data());
    re.resize(nG);
    im.resize(nG);
    for (int m = 0; m < nG; ++m) {
        double q = 2.0 * M_PI * (double)m / (double)n;
        std::complex<double> tmp = std::exp(std::complex<double>(0.0, -(order - 1.0) * q));
        std::complex<double> fac(0.0, 0.0);
        for (int k = 1; k < order; ++k) fac += Mn[k] * std::exp(std::complex<double>(0.0, -(double)k * q));
        std::complex<double> b = tmp / fac;
        re[m] = b.real();
        im[m] = b.imag();
    }
}

double erfcinv_host(double y) {
    if (!(y > 0.0 && y < 2.0)) throw std::invalid_argument("erfcinv domain");
    // start from the asymptotic form for small y, then Newton on erfc
    double x;
    if (y < 1.0) {
        double t = std::sqrt(-std::log(y / 2.0));
        x = t;
    } else {
        double t = std::sqrt(-std::log((2.0 - y) / 2.0));
        x = -t;
    }
    for (int it = 0; it < 100; ++it) {
        double f = std::erfc(x) - y;
        double fp = -2.0 / std::sqrt(M_PI) * std::exp(-x * x);
        double dx = f / fp;
        x -= dx;
        if (std::fabs(dx) <= 1e-16 * std::max(1.0, std::fabs(x))) break;
    }
    return x;
}

}  // namespace ofdft
