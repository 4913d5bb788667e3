// Ewald ion-ion energy and forces (src/dftpy/ewald.py:197-864).
//   eta        Get_Best_eta (:256-278), on the host
//   real part  erfc(sqrt(eta) r)/r over all images within Rcut (Energy_real
//              :281-325, Forces_real :541-577), from a cell list
//   reciprocal smooth PME (Energy_rec_PME :786-807, Forces_rec_PME :810-864)
//              or exact structure factors (Energy_rec :449-466, Forces_rec :580-607)
//   correction Energy_corr (:468-482), on the host
//   stress     Stress_real (:609-662) with the real-space sum; Stress_rec_PME
//              (:915-968) or Stress_rec (:719-763) over the mask, G = 0 term
#include "common.cuh"
#include "host_math.h"
#include "pme.cuh"

#include <algorithm>
#include <cstring>

using namespace ofdft;

namespace ofdft {
void frac_coords(const double* lattice, int nat, const double* pos, std::vector<double>& frac);
void lattice_inverse(const double* a, double* inv);
void bspline_tables(const ofdft_grid* g, int order, double** d_re, double** d_im);
}  // namespace ofdft

namespace {

struct CellList {
    int nc[3];
    int K[3];
    const int* start;   // nc0*nc1*nc2 + 1
    const int* atoms;   // atom indices sorted by cell
    const int* cellof;  // cell of each atom
};

// one thread per atom: sum over the (2K+1)^3 neighbour cells (unwrapped, so
// each periodic image of each atom is visited exactly once).  Partials: the
// energy sum, then the six sums of Stress_real (:645-654),
// q_i q_j (2 sqrt(eta/pi) exp(-eta d^2) + erfc(sqrt(eta) d)/d) R_a R_b / d^2.
__global__ void __launch_bounds__(RED_THREADS) k_ewald_real(const double* __restrict__ pos,
                                                            const double* __restrict__ q, int nat,
                                                            const double* __restrict__ lat, CellList cl, double Rcut,
                                                            double eta, double* F, double* partials) {
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nat) {
        const double es = sqrt(eta);
        const double rtol = 0.001;
        const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
        const int c = cl.cellof[i];
        const int c0 = c / (cl.nc[1] * cl.nc[2]), c1 = (c / cl.nc[2]) % cl.nc[1], c2 = c % cl.nc[2];
        double e = 0.0, fx = 0.0, fy = 0.0, fz = 0.0;
        double s6[6] = {0, 0, 0, 0, 0, 0};
        const double sp2 = 2.0 * es / sqrt(M_PI);
        for (int d0 = -cl.K[0]; d0 <= cl.K[0]; ++d0)
            for (int d1 = -cl.K[1]; d1 <= cl.K[1]; ++d1)
                for (int d2 = -cl.K[2]; d2 <= cl.K[2]; ++d2) {
                    const int u0 = c0 + d0, u1 = c1 + d1, u2 = c2 + d2;
                    const int w0 = pmod(u0, cl.nc[0]), w1 = pmod(u1, cl.nc[1]), w2 = pmod(u2, cl.nc[2]);
                    const double n0 = floor((double)u0 / cl.nc[0]), n1 = floor((double)u1 / cl.nc[1]),
                                 n2 = floor((double)u2 / cl.nc[2]);
                    const double tx = n0 * lat[0] + n1 * lat[3] + n2 * lat[6];
                    const double ty = n0 * lat[1] + n1 * lat[4] + n2 * lat[7];
                    const double tz = n0 * lat[2] + n1 * lat[5] + n2 * lat[8];
                    const int cell = (w0 * cl.nc[1] + w1) * cl.nc[2] + w2;
                    for (int p = cl.start[cell]; p < cl.start[cell + 1]; ++p) {
                        const int j = cl.atoms[p];
                        const double dx = xi - (pos[3 * j] + tx), dy = yi - (pos[3 * j + 1] + ty),
                                     dz = zi - (pos[3 * j + 2] + tz);
                        const double d = sqrt(dx * dx + dy * dy + dz * dz);
                        if (d < Rcut && d > rtol) {
                            const double x = es * d;
                            const double ec = erfc(x);
                            e += q[j] * ec / d;
                            const double w = q[j] * (ec / (x * x * x) + 2.0 / sqrt(M_PI) * exp(-x * x) / (x * x));
                            fx += dx * w;
                            fy += dy * w;
                            fz += dz * w;
                            const double ws = q[j] * (sp2 * exp(-eta * d * d) + ec / d) / (d * d);
                            s6[0] += ws * dx * dx;
                            s6[1] += ws * dx * dy;
                            s6[2] += ws * dx * dz;
                            s6[3] += ws * dy * dy;
                            s6[4] += ws * dy * dz;
                            s6[5] += ws * dz * dz;
                        }
                    }
                }
        acc[0] = q[i] * e;
        for (int k = 0; k < 6; ++k) acc[1 + k] = q[i] * s6[k];
        const double e3 = es * es * es;
        F[3 * i] = q[i] * fx * e3;
        F[3 * i + 1] = q[i] * fy * e3;
        F[3 * i + 2] = q[i] * fz * e3;
    }
    block_sum_store<7>(acc, partials);
}

// PME reciprocal energy partials and the force convolution input:
// E = 4 pi/V sum_mask |Q(G) B(G)|^2 exp(-G^2/4 eta)/G^2 (raw FFT, dV factors cancel);
// X = Q(G) |B(G)|^2 exp(-G^2/4 eta)/G^2 / N
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_ewald_rec_pme(const typename Cplx<T>::type* __restrict__ QG,
                                                               typename Cplx<T>::type* X, const double* bre,
                                                               const double* bim, Geo geo, double eta,
                                                               double* partials) {
    double acc[1] = {0.0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        double gg = gsq(geo, i);
        double br, bi;
        barray(bre, bim, geo, i, br, bi);
        double qr = (double)QG[i].x, qi = (double)QG[i].y;
        double sr = qr * br - qi * bi, si = qr * bi + qi * br;
        double inv = (i == 0) ? 0.0 : 1.0 / gg;
        double w = exp(-gg / (4.0 * eta)) * inv;
        if (half_mask(geo, i)) acc[0] += (sr * sr + si * si) * w;
        if (X) {
            double b2 = br * br + bi * bi;
            double f = b2 * w / (double)geo.N;
            X[i].x = (T)(qr * f);
            X[i].y = (T)(qi * f);
        }
    }
    block_sum_store<1>(acc, partials);
}

// exact structure factor S(G) = sum_a q_a exp(-i G.R_a) and the energy sum
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_ewald_rec_exact(const double* __restrict__ pos,
                                                                 const double* __restrict__ q, int nat, Geo geo,
                                                                 double eta, double* S, double* partials) {
    double acc[1] = {0.0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        double sr = 0.0, si = 0.0;
        for (int a = 0; a < nat; ++a) {
            double ph = gx * pos[3 * a] + gy * pos[3 * a + 1] + gz * pos[3 * a + 2];
            double sn, cs;
            sincos(ph, &sn, &cs);
            sr += q[a] * cs;
            si -= q[a] * sn;
        }
        S[2 * i] = sr;
        S[2 * i + 1] = si;
        double inv = (i == 0) ? 0.0 : 1.0 / gg;
        if (half_mask(geo, i)) acc[0] += (sr * sr + si * si) * exp(-gg / (4.0 * eta)) * inv;
    }
    block_sum_store<1>(acc, partials);
}

// Reciprocal stress sums over the mask (Stress_rec_PME :937-950, Stress_rec
// :733-751): |S(G)|^2 exp(-G^2/4 eta)/G^2 (2 g_i g_j/G^2 (1 + G^2/4 eta) - delta_ij)
// with S = FFT(Q) B (PME, raw transform) or the exact structure factor.
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_ewald_stress_rec(const typename Cplx<T>::type* __restrict__ QG,
                                                                  const double* __restrict__ S, const double* bre,
                                                                  const double* bim, Geo geo, double eta,
                                                                  double* partials) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        if (!half_mask(geo, i)) continue;
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        double sr, si;
        if (QG) {
            double br, bi;
            barray(bre, bim, geo, i, br, bi);
            const double qr = (double)QG[i].x, qi = (double)QG[i].y;
            sr = qr * br - qi * bi;
            si = qr * bi + qi * br;
        } else {
            sr = S[2 * i];
            si = S[2 * i + 1];
        }
        const double inv = (i == 0) ? 0.0 : 1.0 / gg;
        const double w = (sr * sr + si * si) * exp(-gg / (4.0 * eta)) * inv;
        const double f = 2.0 * inv * (1.0 + gg / (4.0 * eta));
        const double g[3] = {gx, gy, gz};
        int k = 0;
        for (int a = 0; a < 3; ++a)
            for (int b = a; b < 3; ++b, ++k) acc[k] += w * (g[a] * g[b] * f - (a == b ? 1.0 : 0.0));
    }
    block_sum_store<6>(acc, partials);
}

constexpr int kChunk = 8;

// exact reciprocal forces for a chunk of atoms:
// F_a = 8 pi/V sum_mask G (Re s_a Im S - Im s_a Re S) exp(-G^2/4eta)/G^2, s_a = q_a e^{-iG.R_a}
__global__ void __launch_bounds__(RED_THREADS) k_ewald_force_exact(const double* __restrict__ pos,
                                                                   const double* __restrict__ q, const double* S,
                                                                   int a0, int na, Geo geo, double eta,
                                                                   double* partials) {
    double acc[3 * kChunk];
    for (int t = 0; t < 3 * kChunk; ++t) acc[t] = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < geo.Nc; i += stride) {
        if (!half_mask(geo, i)) continue;
        double gx, gy, gz, gg;
        gvec(geo, i, gx, gy, gz, gg);
        double inv = (i == 0) ? 0.0 : 1.0 / gg;
        double w = exp(-gg / (4.0 * eta)) * inv;
        double Sr = S[2 * i], Si = S[2 * i + 1];
        for (int t = 0; t < na; ++t) {
            const int a = a0 + t;
            double ph = gx * pos[3 * a] + gy * pos[3 * a + 1] + gz * pos[3 * a + 2];
            double sn, cs;
            sincos(ph, &sn, &cs);
            double sr = q[a] * cs, si = -q[a] * sn;
            double den = (sr * Si - si * Sr) * w;
            acc[3 * t] += gx * den;
            acc[3 * t + 1] += gy * den;
            acc[3 * t + 2] += gz * den;
        }
    }
    block_sum_store<3 * kChunk>(acc, partials);
}

double best_eta(double precision, double gmax, const std::vector<double>& q) {
    double q2 = 0.0;
    for (double x : q) q2 += x * x;
    const double nat = (double)q.size();
    double eta = 1.6;
    for (int it = 0; it < 100000; ++it) {
        double up = 4.0 * M_PI * nat * q2 * std::sqrt(eta / M_PI) * std::erfc(gmax / 2.0 * std::sqrt(1.0 / eta));
        if (up < precision) return eta;
        eta = eta - 0.01;
        if (eta <= 0.0) break;
    }
    set_error("Ewald: no eta satisfies precision %g", precision);
    throw Error{OFDFT_EINVAL};
}

template <typename T>
void ewald_t(ofdft_grid* g, int nat, const double* pos, const double* charges, double precision, int pme, int order,
             double* out_energy, double* forces, double* out_eta, double* stress, cudaStream_t st) {
    using C = typename Cplx<T>::type;
    std::vector<double> q(charges, charges + nat);
    // gmax = sqrt(2 ecut), ecut from the grid spacing (grid.py:363-366, :722-723)
    double lengths[3], sp[3];
    for (int d = 0; d < 3; ++d) {
        const double* a = g->lattice + 3 * d;
        lengths[d] = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        sp[d] = 0.5 * (lengths[d] / g->nr[d] + lengths[d] / (g->nr[d] - 1));
    }
    double spmax = std::max(sp[0], std::max(sp[1], sp[2]));
    double ecut = M_PI * M_PI / (2 * spmax * spmax);
    const double gmax = std::sqrt(2.0 * ecut);
    const double eta = best_eta(precision, gmax, q);
    if (out_eta) *out_eta = eta;
    const double Rcut = erfcinv_host(precision / 3.0) / std::sqrt(eta);

    // ---- correction (ewald.py:468-482)
    double q2 = 0.0, qs = 0.0;
    for (double x : q) {
        q2 += x * x;
        qs += x;
    }
    const double e_corr = -std::sqrt(eta / M_PI) * q2 - 4.0 * M_PI * (1.0 / (4.0 * eta * g->volume) / 2.0) * qs * qs;

    // ---- real space on a cell list
    std::vector<double> frac;
    frac_coords(g->lattice, nat, pos, frac);
    std::vector<double> wpos(3 * (size_t)nat);
    for (int a = 0; a < nat; ++a)
        for (int k = 0; k < 3; ++k)
            wpos[3 * a + k] = frac[3 * a] * g->lattice[k] + frac[3 * a + 1] * g->lattice[3 + k] +
                              frac[3 * a + 2] * g->lattice[6 + k];
    // perpendicular widths w_d = V / |a_e x a_f|
    const double* L = g->lattice;
    auto cross_norm = [&](int e, int f) {
        const double* u = L + 3 * e;
        const double* v = L + 3 * f;
        double cx = u[1] * v[2] - u[2] * v[1], cy = u[2] * v[0] - u[0] * v[2], cz = u[0] * v[1] - u[1] * v[0];
        return std::sqrt(cx * cx + cy * cy + cz * cz);
    };
    double wd[3] = {g->volume / cross_norm(1, 2), g->volume / cross_norm(0, 2), g->volume / cross_norm(0, 1)};
    CellList cl;
    for (int d = 0; d < 3; ++d) {
        cl.nc[d] = std::max(1, std::min(64, (int)std::floor(wd[d] / Rcut)));
        cl.K[d] = (int)std::ceil(Rcut * cl.nc[d] / wd[d]);
    }
    const int ncell = cl.nc[0] * cl.nc[1] * cl.nc[2];
    std::vector<int> cellof(nat), start(ncell + 1, 0), order_atoms(nat);
    for (int a = 0; a < nat; ++a) {
        int c[3];
        for (int d = 0; d < 3; ++d) c[d] = std::min(cl.nc[d] - 1, (int)(frac[3 * a + d] * cl.nc[d]));
        cellof[a] = (c[0] * cl.nc[1] + c[1]) * cl.nc[2] + c[2];
        start[cellof[a] + 1]++;
    }
    for (int c = 0; c < ncell; ++c) start[c + 1] += start[c];
    {
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int a = 0; a < nat; ++a) order_atoms[fill[cellof[a]]++] = a;
    }
    Scratch sc;
    double* d_pos = (double*)sc.get("pos", 3 * (size_t)nat * sizeof(double));
    double* d_q = (double*)sc.get("q", (size_t)nat * sizeof(double));
    double* d_lat = (double*)sc.get("lat", 9 * sizeof(double));
    int* d_start = (int*)sc.get("start", (ncell + 1) * sizeof(int));
    int* d_atoms = (int*)sc.get("atoms", (size_t)nat * sizeof(int));
    int* d_cellof = (int*)sc.get("cellof", (size_t)nat * sizeof(int));
    double* d_F = (double*)sc.get("F", 3 * (size_t)nat * sizeof(double));
    double* d_Fr = (double*)sc.get("Fr", 3 * (size_t)nat * sizeof(double));
    double* d_frac = (double*)sc.get("frac", 3 * (size_t)nat * sizeof(double));
    double* d_scale = (double*)sc.get("scale", (size_t)nat * sizeof(double));
    double* d_cinv = (double*)sc.get("cinv", 9 * sizeof(double));
    OFDFT_CK(cudaMemcpyAsync(d_pos, wpos.data(), 3 * (size_t)nat * sizeof(double), cudaMemcpyHostToDevice, st));
    OFDFT_CK(cudaMemcpyAsync(d_q, q.data(), (size_t)nat * sizeof(double), cudaMemcpyHostToDevice, st));
    OFDFT_CK(cudaMemcpyAsync(d_lat, g->lattice, 9 * sizeof(double), cudaMemcpyHostToDevice, st));
    OFDFT_CK(cudaMemcpyAsync(d_start, start.data(), (ncell + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    OFDFT_CK(cudaMemcpyAsync(d_atoms, order_atoms.data(), (size_t)nat * sizeof(int), cudaMemcpyHostToDevice, st));
    OFDFT_CK(cudaMemcpyAsync(d_cellof, cellof.data(), (size_t)nat * sizeof(int), cudaMemcpyHostToDevice, st));
    OFDFT_CK(cudaMemcpyAsync(d_frac, frac.data(), 3 * (size_t)nat * sizeof(double), cudaMemcpyHostToDevice, st));
    cl.start = d_start;
    cl.atoms = d_atoms;
    cl.cellof = d_cellof;
    const int ablk = (nat + RED_THREADS - 1) / RED_THREADS;
    OFDFT_REQUIRE(ablk <= g->red_blocks * 32, "Ewald: too many atoms for the reduction buffer");
    k_ewald_real<<<ablk, RED_THREADS, 0, st>>>(d_pos, d_q, nat, d_lat, cl, Rcut, eta, d_Fr, g->d_partials);
    OFDFT_LAUNCH_CHECK();
    reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, ablk, 7, 0ull, g->d_results);
    OFDFT_LAUNCH_CHECK();
    OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, 7 * sizeof(double), cudaMemcpyDeviceToHost, st));
    OFDFT_CK(cudaStreamSynchronize(st));
    const double e_real = g->h_results[0] / 2.0;
    double s_real[6];
    for (int k = 0; k < 6; ++k) s_real[k] = g->h_results[1 + k] * (-0.5 / g->volume);
    std::vector<double> Freal(3 * (size_t)nat);
    OFDFT_CK(cudaMemcpyAsync(Freal.data(), d_Fr, 3 * (size_t)nat * sizeof(double), cudaMemcpyDeviceToHost, st));
    OFDFT_CK(cudaStreamSynchronize(st));

    // ---- reciprocal space
    double e_rec = 0.0;
    double s_rec[6] = {0, 0, 0, 0, 0, 0};
    std::vector<double> Frec(3 * (size_t)nat, 0.0);
    const size_t cb = g->cplx_bytes(), rb = g->real_bytes();
    if (pme) {
        OFDFT_REQUIRE(g->nr[0] >= order && g->nr[1] >= order && g->nr[2] >= order,
                      "PME needs at least %d grid points per axis", order);
        double *bre = nullptr, *bim = nullptr;
        bspline_tables(g, order, &bre, &bim);
        T* Q = (T*)sc.get("Q", rb);
        C* QG = (C*)sc.get("QG", cb);
        C* X = forces ? (C*)sc.get("X", cb) : nullptr;
        const PmeTiles tiles = pme_tiles_build(sc, "pme_", frac.data(), nullptr, nat, order, g->nr, st);
        pme_spread<T>(tiles, d_frac, nullptr, d_q, g->geo, Q, rb, st);
        g->exec_r2c(Q, QG, 1, st);
        k_ewald_rec_pme<T><<<g->red_blocks, RED_THREADS, 0, st>>>(QG, X, bre, bim, g->geo, eta, g->d_partials);
        OFDFT_LAUNCH_CHECK();
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 1, 0ull, g->d_results);
        OFDFT_LAUNCH_CHECK();
        OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        e_rec = 4.0 * M_PI * g->h_results[0] / g->volume;
        if (stress) {
            k_ewald_stress_rec<T><<<g->red_blocks, RED_THREADS, 0, st>>>(QG, nullptr, bre, bim, g->geo, eta,
                                                                         g->d_partials);
            OFDFT_LAUNCH_CHECK();
            reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 6, 0ull, g->d_results);
            OFDFT_LAUNCH_CHECK();
            OFDFT_CK(cudaMemcpyAsync(s_rec, g->d_results, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
            OFDFT_CK(cudaStreamSynchronize(st));
        }
        if (forces) {
            T* conv = (T*)sc.get("conv", rb);
            g->exec_c2r(X, conv, 1, st);
            double cinv[9];
            lattice_inverse(g->lattice, cinv);
            std::vector<double> scale(nat);
            for (int a = 0; a < nat; ++a) scale[a] = -q[a] * 4.0 * M_PI / g->dV;
            OFDFT_CK(cudaMemcpyAsync(d_cinv, cinv, 9 * sizeof(double), cudaMemcpyHostToDevice, st));
            OFDFT_CK(cudaMemcpyAsync(d_scale, scale.data(), (size_t)nat * sizeof(double), cudaMemcpyHostToDevice, st));
            k_pme_gather<T><<<nat, 256, 0, st>>>(d_frac, nullptr, order, g->geo, conv, d_cinv, d_scale, d_F);
            OFDFT_LAUNCH_CHECK();
            OFDFT_CK(cudaMemcpyAsync(Frec.data(), d_F, 3 * (size_t)nat * sizeof(double), cudaMemcpyDeviceToHost, st));
            OFDFT_CK(cudaStreamSynchronize(st));
        }
        cudaFree(bre);
        cudaFree(bim);
    } else {
        double* S = (double*)sc.get("S", (size_t)g->Nc * 2 * sizeof(double));
        k_ewald_rec_exact<T><<<g->red_blocks, RED_THREADS, 0, st>>>(d_pos, d_q, nat, g->geo, eta, S, g->d_partials);
        OFDFT_LAUNCH_CHECK();
        reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 1, 0ull, g->d_results);
        OFDFT_LAUNCH_CHECK();
        OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, sizeof(double), cudaMemcpyDeviceToHost, st));
        OFDFT_CK(cudaStreamSynchronize(st));
        e_rec = 4.0 * M_PI * g->h_results[0] / g->volume;
        if (stress) {
            k_ewald_stress_rec<T><<<g->red_blocks, RED_THREADS, 0, st>>>(nullptr, S, nullptr, nullptr, g->geo, eta,
                                                                         g->d_partials);
            OFDFT_LAUNCH_CHECK();
            reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 6, 0ull, g->d_results);
            OFDFT_LAUNCH_CHECK();
            OFDFT_CK(cudaMemcpyAsync(s_rec, g->d_results, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
            OFDFT_CK(cudaStreamSynchronize(st));
        }
        if (forces) {
            for (int a0 = 0; a0 < nat; a0 += kChunk) {
                const int na = std::min(kChunk, nat - a0);
                k_ewald_force_exact<<<g->red_blocks, RED_THREADS, 0, st>>>(d_pos, d_q, S, a0, na, g->geo, eta,
                                                                           g->d_partials);
                OFDFT_LAUNCH_CHECK();
                reduce_finalize<<<1, RED_THREADS, 0, st>>>(g->d_partials, g->red_blocks, 3 * kChunk, 0ull,
                                                           g->d_results);
                OFDFT_LAUNCH_CHECK();
                OFDFT_CK(cudaMemcpyAsync(g->h_results, g->d_results, 3 * kChunk * sizeof(double),
                                         cudaMemcpyDeviceToHost, st));
                OFDFT_CK(cudaStreamSynchronize(st));
                for (int t = 0; t < na; ++t)
                    for (int c = 0; c < 3; ++c) Frec[3 * (a0 + t) + c] = g->h_results[3 * t + c] * 8.0 * M_PI / g->volume;
            }
        }
    }
    out_energy[0] = e_corr + e_real + e_rec;
    out_energy[1] = e_real;
    out_energy[2] = e_rec;
    out_energy[3] = e_corr;
    if (forces)
        for (size_t k = 0; k < 3 * (size_t)nat; ++k) forces[k] = Freal[k] + Frec[k];
    if (stress) {
        // both reciprocal forms reduce to 4 pi / V^2 times the mask sums (the PME
        // form's 2 x 2 pi / V^2 / dV^2 with the dV^2 of its transforms); the G = 0
        // term (sum q)^2 4 pi / (8 eta V^2) sits on the diagonal
        const double V2 = g->volume * g->volume;
        const double sg0 = qs * qs * 4.0 * M_PI * (1.0 / (4.0 * eta * V2) / 2.0);
        static const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {0, 1, 2, 1, 2, 2};
        for (int k = 0; k < 6; ++k) {
            double v = s_real[k] + s_rec[k] * 4.0 * M_PI / V2;
            if (I[k] == J[k]) v += sg0;
            stress[3 * I[k] + J[k]] = stress[3 * J[k] + I[k]] = v;
        }
    }
}

}  // namespace

// both precisions run the Ewald sums in float64: an FP32 grid gets a float64
// twin for the PME mesh, built for this call only
static void ewald_any(ofdft_grid* g, int nat, const double* pos, const double* charges, double precision, int pme,
               int bspline_order, double* out_energy, double* forces, double* out_eta, double* stress,
               cudaStream_t st) {
    OFDFT_REQUIRE(g && pos && charges && nat >= 1, "ofdft_ewald: bad argument");
    OFDFT_REQUIRE(precision > 0.0 && precision < 1.0, "ofdft_ewald: precision must be in (0, 1)");
    OFDFT_REQUIRE(!pme || (bspline_order >= 3 && bspline_order <= kMaxOrder), "B-spline order must be 3..%d",
                  kMaxOrder);
    if (g->prec == OFDFT_F64) {
        ewald_t<double>(g, nat, pos, charges, precision, pme, bspline_order, out_energy, forces, out_eta, stress, st);
        return;
    }
    ofdft_grid* gd = nullptr;
    int rc = ofdft_grid_create(g->nr, g->lattice, OFDFT_F64, &gd);
    if (rc != OFDFT_OK) throw Error{rc};
    try {
        ewald_t<double>(gd, nat, pos, charges, precision, pme, bspline_order, out_energy, forces, out_eta, stress, st);
    } catch (...) {
        ofdft_grid_destroy(gd);
        throw;
    }
    ofdft_grid_destroy(gd);
}

extern "C" int ofdft_ewald(ofdft_grid* g, int nat, const double* pos, const double* charges, double precision, int pme,
                           int bspline_order, double* out_energy, double* forces, double* out_eta, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(out_energy, "ofdft_ewald: null energy output");
        ewald_any(g, nat, pos, charges, precision, pme, bspline_order, out_energy, forces, out_eta, nullptr,
                  (cudaStream_t)s);
    });
}

extern "C" int ofdft_ewald_stress(ofdft_grid* g, int nat, const double* pos, const double* charges, double precision,
                                  int pme, int bspline_order, double* stress, double* out_eta, ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(stress, "ofdft_ewald_stress: null stress output");
        double energy[4];
        ewald_any(g, nat, pos, charges, precision, pme, bspline_order, energy, nullptr, out_eta, stress,
                  (cudaStream_t)s);
    });
}
