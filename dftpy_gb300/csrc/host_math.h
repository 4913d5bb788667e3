// Host-side numerics shared by the evaluator, pseudopotential and Ewald code.
#pragma once
#include <vector>

namespace ofdft {

// Interpolating cubic spline with not-a-knot end conditions through (x_i, y_i),
// i.e. the spline FITPACK's splrep(x, y, k=3, s=0) returns (its interior knots
// are x_2..x_{n-3}).  Stored per data interval i as y = c0 + c1 u + c2 u^2 + c3 u^3,
// u = x - x_i.  x must be strictly increasing, n >= 4.
struct CubicSpline {
    std::vector<double> x;
    std::vector<double> c;  // 4 per interval, (n-1) intervals
    void fit(const std::vector<double>& x, const std::vector<double>& y);
    int interval(double xv) const;
    double eval(double xv) const;
    double deriv(double xv) const;
    // Adjoint of fit(): given dL/dc (4 per interval) return dL/dy (n values).
    // The fit is linear in y, so this is the transpose of the data-to-coefficient map.
    std::vector<double> adjoint(const std::vector<double>& gc) const;
};

// Inverse Lindhard function F(eta; lambda, mu) with the reference's four
// branches (src/dftpy/functional/kedf/kernel.py:14-136).
double lindhard(double eta, double lbda, double mu);

// MGP kernel table on the points eta (src/dftpy/functional/kedf/kernel.py:267-322,
// serial): sym 0 none, 1 arithmetic (averaged with the WT table), 2 geometric.
std::vector<double> mgp_kernel_table(const std::vector<double>& eta, int maxpoints, int sym);

// k_F bound rule of the density-dependent kernel (src/dftpy/functional/kedf/lwt.py:36-79).
// state_set/state_min/state_max carry the saved bounds between calls.
void guess_kf_bound(double kf_l, double kf_r, bool fixed_min, double kfmin_in, bool fixed_max, double kfmax_in,
                    bool& state_set_min, double& state_min, bool& state_set_max, double& state_max,
                    double& out_min, double& out_max);

// k_F nodes (lwt.py:174-190): nsp uniform nodes, spacing delta, or ratio.
std::vector<double> kf_nodes(double kfMin, double kfMax, int nsp, double delta, double ratio);

// k_F nodes of the HC kernels (get_kflist, hc.py:16-66): bounds snapped to powers
// of ratio (kf0 = 1), kept from the saved state when they moved little; the
// state is updated.
std::vector<double> hc_kf_nodes(double kf_l, double kf_r, bool fixed_min, double kfmin_in, bool fixed_max,
                                double kfmax_in, bool& set_min, double& st_min, bool& set_max, double& st_max,
                                double ratio, int nsp, double delta);

// Cardinal B-spline values of CBspline.calc_Mn (src/dftpy/ewald.py:63-82):
// out[n] = M_order(x + n - 1), n = 1..order (out has order_full+1 entries).
void bspline_mn(double x, int order, int order_full, double* out);

// exp(-i (order-1) q) / sum_k M_order(k) exp(-i k q), q = 2 pi m / n (ewald.py:84-101)
void bspline_bm(int n, int nG, int order, std::vector<double>& re, std::vector<double>& im);

// erfc^{-1}(y) for 0 < y < 2 by Newton iteration on erfc.
double erfcinv_host(double y);

}  // namespace ofdft
