/*
 * ofdft.h -- C ABI of the GB300 (sm_103a) orbital-free DFT hot path.
 *
 * A drop-in device backend for the energy + potential (E+V) evaluation of
 * DFTpy's total density functional and the density optimisation built on it.
 * Every entry point is extern "C", takes plain pointers, sizes and a CUDA
 * stream, returns an int status (0 = OK) and never throws.  Device pointers
 * are caller-owned (the Python layer passes torch CUDA tensors); handles own
 * cuFFT plans, tables and scratch.  A handle is not thread-safe: use one per
 * host thread / stream.  On error, ofdft_last_error() returns a message.
 *
 * Units are atomic (Hartree, Bohr); densities in e/Bohr^3.  Real fields are
 * C-ordered (n0, n1, n2) arrays; reciprocal fields are the half-complex
 * (n0, n1, n2/2+1) arrays of an R2C transform (the reference's default
 * "gfull=False" grid).  Precision OFDFT_F64 computes in float64 throughout;
 * OFDFT_F32 ("FP32-mixed") stores grids and runs FFTs and pointwise work in
 * float32; energy / electron-count / dot-product sums run per thread in
 * compensated (Kahan) float32 and across threads in float64.
 *
 * Reference interfaces each group replaces are cited as
 * path:line within Quantum-MultiScale/DFTpy.
 */
#ifndef OFDFT_H
#define OFDFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ofdft_grid ofdft_grid;         /* grid + FFT plans + scratch   */
typedef struct ofdft_eval ofdft_eval;         /* configured total functional  */
typedef void* ofdft_stream;                   /* a cudaStream_t (NULL = legacy default) */

enum { OFDFT_OK = 0, OFDFT_EINVAL = 1, OFDFT_ECUDA = 2, OFDFT_ECUFFT = 3, OFDFT_ENOMEM = 4,
       OFDFT_ESTATE = 5 };
enum { OFDFT_F64 = 0, OFDFT_F32 = 1 };
enum { OFDFT_CALC_E = 1, OFDFT_CALC_V = 2 };

/* energy slots written by ofdft_eval_compute (Hartree) */
enum { OFDFT_E_TF = 0, OFDFT_E_VW, OFDFT_E_NL, OFDFT_E_XC, OFDFT_E_H, OFDFT_E_PP, OFDFT_E_II,
       OFDFT_E_TOTAL, OFDFT_E_NELEC, OFDFT_E_GGA, OFDFT_E_EXT, OFDFT_E_DTTF, OFDFT_NE };
/* stress tensors written by ofdft_eval_stress, 9 doubles (3 x 3, row-major) each */
enum { OFDFT_S_TF = 0, OFDFT_S_VW, OFDFT_S_NL, OFDFT_S_XC, OFDFT_S_H, OFDFT_S_GGA, OFDFT_NS };

/* ---------------------------------------------------------------- errors */
const char* ofdft_last_error(void);
const char* ofdft_version(void);

/* ------------------------------------------------------------------ grid
 * DirectGrid / ReciprocalGrid (src/dftpy/grid.py:8-60, :384-415, :480-620):
 * lattice rows are the lattice vectors (Bohr).  G vectors are computed from
 * the index and the reciprocal lattice on the fly, never stored. */
int ofdft_grid_create(const int nr[3], const double lattice[9], int precision, ofdft_grid** out);
void ofdft_grid_destroy(ofdft_grid* g);
int ofdft_grid_info(const ofdft_grid* g, int nr[3], double* volume, double* dV, int* precision);

/* DirectField.fft (src/dftpy/field.py:413-430): out = rfftn(in) * dV.
 * ReciprocalField.ifft (field.py:779-804): out = irfftn(in) / dV.  The input of
 * ofdft_ifft is not modified (it is copied to scratch first). */
int ofdft_fft(ofdft_grid* g, const void* in_real, void* out_cplx, ofdft_stream s);
int ofdft_ifft(ofdft_grid* g, const void* in_cplx, void* out_real, ofdft_stream s);
/* Fourier interpolation of a real field from grid src to grid dst of the same
 * cell (grid_map_data / grid_map_index, src/dftpy/utils/utils.py:50-128): the
 * source coefficients keep their frequencies, those the destination lacks are
 * dropped, the rest are zero.  dst must be finer or coarser on every axis.
 * floor_value: values below it are raised to it (field2distrib's tol,
 * utils.py:265), or -INFINITY for none.  in: src precision; out: dst field. */
int ofdft_grid_map(ofdft_grid* src, ofdft_grid* dst, const void* in, void* out, double floor_value,
                   ofdft_stream s);

/* Reductions over a real field in float64 with a fixed summation order
 * (mp.einsum/vsum, src/dftpy/mpi/mpi.py:199-246).  out[0] = sum(a*b) (b may be
 * NULL: sum(a)).  ofdft_dot3: sum(a*b*c). */
int ofdft_dot(ofdft_grid* g, const void* a, const void* b, double* out, ofdft_stream s);
int ofdft_dot3(ofdft_grid* g, const void* a, const void* b, const void* c, double* out, ofdft_stream s);

/* The same float64 reduction without a grid handle and without any allocation,
 * for callers that cannot allocate device memory where they need it (inside
 * an allocator or memory-pool hook, in loops that forbid allocation after
 * start-up, or when a framework pool has reserved all device memory).  This
 * entry point has no counterpart in the reference.  out_dev[0] = sum(a*b) (b
 * may be NULL: sum(a)) over n elements of the given precision, written to
 * device memory in stream order.  Its scratch is a 32 KiB static device array
 * (4096 block partials), so n is limited to 67,108,864 (OFDFT_EINVAL beyond).
 * The first call on a device looks the array up and loads this entry point's
 * kernels (under lazy module loading that load takes device memory), so make
 * it at start-up, before a pool reserves the device's memory and before any
 * stream capture; calls that overlap on the GPU share the array and race. */
int ofdft_dot_noalloc(const void* a, const void* b, long long n, int precision, double* out_dev, ofdft_stream s);

/* ------------------------------------------------------ total functional
 * Configuration of the terms of TotalFunctional (src/dftpy/functional/
 * total_functional.py:49-146) and the KEDF dispatcher (kedf/__init__.py:27-69,
 * :124-191).  kedf_terms is a bit set of OFDFT_KE_*. */
enum { OFDFT_KE_TF = 1, OFDFT_KE_VW = 2, OFDFT_KE_WT = 4, OFDFT_KE_LWT = 8, OFDFT_KE_GGA = 16,
       OFDFT_KE_DTTF = 32 /* finite-temperature TF correction TTF (kedf/tf.py:83-204), tf_temperature */ };
/* enhancement-factor formulas of the GGA kinetic functionals (kedf/gga.py:18-586);
 * a named functional of the reference's GGA_KEDF_list (:587-643) is a formula plus
 * its parameters, e.g. LC94 = PW91 with its own six, REVAPBEK = PBE with (1.245, 0.23889) */
enum { OFDFT_GGA_LKT = 0, OFDFT_GGA_LKTVW, OFDFT_GGA_DK, OFDFT_GGA_LLP, OFDFT_GGA_OL, OFDFT_GGA_THAK,
       OFDFT_GGA_B86A, OFDFT_GGA_B86B, OFDFT_GGA_DK87, OFDFT_GGA_PW86, OFDFT_GGA_PW91O, OFDFT_GGA_PW91,
       OFDFT_GGA_LG94, OFDFT_GGA_P92, OFDFT_GGA_PBE, OFDFT_GGA_P82, OFDFT_GGA_VJKS00, OFDFT_GGA_VT84F,
       OFDFT_GGA_TFVW, OFDFT_GGA_STV, OFDFT_GGA_PBE2M, OFDFT_GGA_PG,
       /* Laplacian-level (meta-GGA) formulas of MGGA_KEDF_list (gga.py:645-650): F(s, q)
        * with q = lap(rho) / (TKF0^2 rho^(5/3)); no stress (gga.py:1313-1314) */
       OFDFT_GGA_GE2, OFDFT_GGA_GE4, OFDFT_GGA_PGSL, OFDFT_GGA_PGSLR, OFDFT_GGA_NFORMULAS };
enum { OFDFT_INTERP_LINEAR = 0, OFDFT_INTERP_HERMITE = 1 };
/* k_F-node kernel pipeline: AUTO takes FUSED where it applies (float32 grid,
 * the LWT family, every axis a power of two in 32..256, the last axis up to
 * 512; linear or cubic Hermite interpolation) and CUFFT otherwise; FUSED fails
 * with OFDFT_EINVAL where it does not apply.  FUSED folds the node kernel, the
 * interpolation and the pot2 sum into the library's own tile FFTs; CUFFT runs
 * them as separate passes around batched cuFFT transforms.  Both compute the
 * same quantities.  FUSED_SPLIT (grids with n1 = n2 = 256 and the linear
 * interpolation only) is FUSED with the axis-1 transform of both
 * chains factored as radix 8 x 32 between their column and row passes, so
 * neither chain has an axis-1 plane pass and each node plane crosses HBM twice;
 * it moves half the DRAM bytes of FUSED but runs slower on GB300 (its column
 * tiles take a whole SM each), so AUTO does not take it. */
enum { OFDFT_LWT_PIPE_AUTO = 0, OFDFT_LWT_PIPE_CUFFT = 1, OFDFT_LWT_PIPE_FUSED = 2, OFDFT_LWT_PIPE_FUSED_SPLIT = 3 };
/* kernel table of the k_F-node kernel (lwt.py:535-548): the WT table
 * (kernel.py:344-352, LWT) or the MGP table (kernel.py:267-322; LMGP, and with
 * the arithmetic / geometric symmetrisation LMGPA / LMGPG, lwt.py:571-578) */
enum { OFDFT_LWT_KERNEL_WT = 0, OFDFT_LWT_KERNEL_MGP = 1, OFDFT_LWT_KERNEL_MGPA = 2, OFDFT_LWT_KERNEL_MGPG = 3,
       OFDFT_LWT_KERNEL_USER = 4 /* values from ofdft_eval_set_lwt_table */ };
/* the k_F-node family: LWT (lwt.py:82-341) or HC (hc.py:68-331: k_F = F(s) (3 pi^2 rho)^(1/3)
 * with F from gga_formula/gga_params, nodes by get_kflist, kernel T(q/2k)/(2k)^3, Hermite
 * interpolation, and the gradient terms of dk_F/drho in the potential) */
enum { OFDFT_LWT_FAMILY_LWT = 0, OFDFT_LWT_FAMILY_HC = 1 };

/* Configuration of one evaluator.  Bindings in other languages must mirror
 * this struct member for member; struct_size guards against a stale mirror:
 * ofdft_config_init (or ofdft_config_default) sets it to sizeof(ofdft_config),
 * and ofdft_eval_create refuses a config whose struct_size differs. */
typedef struct {
    unsigned int struct_size; /* sizeof(ofdft_config) of the library: set by ofdft_config_init */
    int    kedf_terms;
    double tf_x;              /* TF prefactor x (kedf/tf.py:66)                    */
    double vw_y;              /* vW prefactor y (kedf/vw.py:115)                   */
    /* Wang-Teter nonlocal term (kedf/wt.py:109-132, kernel.py:325-334)           */
    double wt_alpha, wt_beta, wt_x;
    double wt_rho0;           /* <= 0: mean density of each call (wt.py:112-113)   */
    /* density-dependent kernel table, LWT family (kedf/lwt.py:82-341, :502-568)  */
    double lwt_alpha, lwt_beta, lwt_x;
    int    lwt_nsp;           /* > 0: nsp uniform nodes (lwt.py:174-181)          */
    double lwt_delta;         /* > 0 and nsp <= 0: node spacing (lwt.py:182-184)  */
    double lwt_ratio;         /* otherwise: geometric node ratio (lwt.py:185-188) */
    int    lwt_kdd;           /* 1, 2 or 3 (derivative terms kept)                */
    int    lwt_interp;        /* OFDFT_INTERP_*                                   */
    double lwt_etamax;        /* table range (default 50)                         */
    int    lwt_neta;          /* table points (default 50000)                     */
    double lwt_kfmin, lwt_kfmax; /* fixed k_F bounds, or NaN for the adaptive rule */
    double lwt_ldw;           /* low-density weight exponent (default 1/6)        */
    int    lwt_max_batch;     /* nodes per batched FFT pass (0 = automatic)       */
    int    xc_lda;            /* built-in LDA, Slater + PZ81 (xc/semilocal_xc.py:283-341) */
    int    hartree;           /* Hartree (functional/hartree.py:24-45)             */
    int    pseudo;            /* add the local pseudopotential set by ofdft_eval_set_vloc */
    double ewald_energy;      /* ion-ion energy added to the total (0 = none)     */
    int    lwt_pipeline;      /* OFDFT_LWT_PIPE_*: how the k_F-node kernel runs   */
    int    lwt_kernel;        /* OFDFT_LWT_KERNEL_*: the kernel table              */
    int    lwt_maxpoints;     /* MGP tables: points of the t integral (default 1000) */
    /* GGA kinetic functional (kedf/gga.py:1212-1325), with OFDFT_KE_GGA              */
    int    gga_formula;       /* OFDFT_GGA_*                                       */
    int    gga_nparams;       /* parameters in gga_params (1..8)                   */
    double gga_params[8];
    double gga_remove_vw;     /* gga_remove_vw: vW share subtracted from F (0: none) */
    int    lwt_family;        /* OFDFT_LWT_FAMILY_*                                */
    int    external;          /* add the external potential set by ofdft_eval_set_external */
    double vw_sigma;          /* > 0: vW Laplacian times exp(-G^2 sigma^2/4) (kedf/vw.py:45-48) */
    double gga_sigma;         /* > 0: GGA gradient times exp(-G^2 sigma^2/2), the
                                 'supersmooth' gradient (gga.py:1246-1250, field.py:229-262) */
    int    wte;               /* with TF and WT: WTE (kedf/wte.py:15-57), E = E_TF exp(E_WT/E_TF)
                                 and V = exp(E_WT/E_TF)((1 - E_WT/E_TF) V_TF + V_WT), reported
                                 in OFDFT_E_NL (OFDFT_E_TF = 0) */
    /* kernel of the density-independent nonlocal term (OFDFT_KE_WT): OFDFT_LWT_KERNEL_WT
     * (Lindhard, kernel.py:325-334) or the MGP kernels at rho0 (kedf/mgp.py:15-119,
     * kernel.py:251-322): OFDFT_LWT_KERNEL_MGP/MGPA/MGPG, with wt_maxpoints t points and
     * the lump correction MGPOmegaE (kernel.py:408-440) */
    int    wt_kernel;
    int    wt_maxpoints;      /* default 1000                                        */
    int    wt_lump;           /* 0 none; 1 a = lump[0] / Ne^(2/3) = b; 2 a, b = lump[0..1] */
    double wt_lump_abc[3];    /* a, b, c (c = 1 by default)                          */
    int    wt_revke;          /* 1: erf(c G^2)^2 (MGP, MGPA, MGPG); 0: 3/5 erf(c |G|)^2 (MGP0) */
    double tf_temperature;    /* OFDFT_KE_DTTF: the temperature (Hartree)              */
    int    tf_temp_old;       /* 1: the energy of TemperatureTFEnergy_old (temperature0) */
} ofdft_config;

/* sizeof(ofdft_config) in this library; a binding compares it with the size of
 * its own mirror before it passes one in. */
size_t ofdft_config_size(void);
/* Defaults of every member (the reference's defaults) and struct_size.
 * caller_size is the size of the caller's struct: when it differs from
 * ofdft_config_size() nothing is written and OFDFT_EINVAL is returned, so a
 * stale binding fails here instead of being written past. */
int ofdft_config_init(ofdft_config* c, size_t caller_size);
/* The same without the size check (the caller's struct must be this header's). */
void ofdft_config_default(ofdft_config* c);

int ofdft_eval_create(ofdft_grid* g, const ofdft_config* cfg, ofdft_eval** out);
void ofdft_eval_destroy(ofdft_eval* e);
/* Copy a real-space local pseudopotential (device pointer, grid precision) into
 * the evaluator (LocalPseudo._vreal, src/dftpy/functional/pseudo/__init__.py:219-234). */
int ofdft_eval_set_vloc(ofdft_eval* e, const void* vloc_dev, ofdft_stream s);
int ofdft_eval_set_ewald(ofdft_eval* e, double energy);
/* Copy a frozen external potential (device pointer, grid precision) into the
 * evaluator: ExternalPotential (functional/external_potential.py:7-40), energy
 * dV sum(v rho) in OFDFT_E_EXT, v added to the potential.  OE-SCF freezes the
 * embedding potential this way (optimization/scf.py:83-96). */
int ofdft_eval_set_external(ofdft_eval* e, const void* v_dev, ofdft_stream s);

/* TotalFunctional.compute(rho, calcType) (total_functional.py:107-146).
 * rho: device field (not modified).  v_out: device field for the total
 * potential (required with OFDFT_CALC_V, may be NULL otherwise).  energies:
 * host array of OFDFT_NE doubles (per-term energies, total, electron count). */
int ofdft_eval_compute(ofdft_eval* e, const void* rho, void* v_out, unsigned calc,
                       double* energies, ofdft_stream s);

/* ---- density mixing of OE-SCF (src/dftpy/mixer/mixer.py:8-169, pulay.py:8-120,
 * linear.py:4-35).  Fields are device arrays in the grid's precision. */
enum { OFDFT_PRED_NONE = 0, OFDFT_PRED_KERKER = 1, OFDFT_PRED_INVERSE_KERKER = 2, OFDFT_PRED_RESTA = 3 };
#define OFDFT_MIX_MAXM 8

/* PulayMixer history step (pulay.py:53-68, :101-102): r = nout - nin; unless
 * first != 0, dn = nin - prev_n and dr = r - prev_r; then prev_n = nin and
 * prev_r = r.  dn and dr may be NULL when first != 0. */
int ofdft_mix_history(ofdft_grid* g, const void* nin, const void* nout, void* prev_n, void* prev_r, void* dn,
                      void* dr, int first, ofdft_stream s);

/* gram[i*nf+j] = sum over points of f_i f_j for nf fields (1..OFDFT_MIX_MAXM+1) in
 * one pass: the Pulay matrix and right-hand side (pulay.py:70-77).  gram: host. */
int ofdft_mix_gram(ofdft_grid* g, const void* const* fields, int nf, double* gram, ofdft_stream s);

typedef struct {
    int    predtype;          /* OFDFT_PRED_*: the G-space matrix (mixer.py:28-40, 72-117) */
    double predcoef[3];       /* [a0 or epsilon, q0, amin or rs]                   */
    int    cutoff;            /* nonzero: above gmax mix linearly (mixer.py:56-70, 136-139) */
    double predecut;          /* Hartree: gmax = 2 predecut, or, below 2, the largest
                                 |G|^2 along the three axes + 2                     */
    double coef;              /* multiplies the residual term (pulay.py:90, linear.py:26) */
    double mask_coef;         /* weight of nout above gmax                          */
    double resw;              /* weight of nout - nin in the residual: 1 for the
                                 mixers, 0 for a residual given as dr[0] with x[0] = 1 */
    int    ns;                /* history terms used, 0..OFDFT_MIX_MAXM              */
    const void* dn[OFDFT_MIX_MAXM];  /* NULL entries add nothing                   */
    const void* dr[OFDFT_MIX_MAXM];
    double x[OFDFT_MIX_MAXM]; /* Pulay coefficients                                 */
} ofdft_mix_args;

/* Mixed density (SpecialPrecondition.compute, mixer.py:126-140, with the Pulay
 * combination of pulay.py:78-92): out = IFFT(FFT(nin + sum x_i dn_i) +
 * M(G) FFT(coef (resw (nout - nin) + sum x_i dr_i))), and FFT((1 - mask_coef) nin +
 * mask_coef nout) where |G|^2 > gmax.  out must not alias nin or nout. */
int ofdft_mix_density(ofdft_grid* g, const void* nin, const void* nout, const ofdft_mix_args* a, void* out,
                      ofdft_stream s);

/* Stress tensors (Ha/Bohr^3) of the evaluator's terms on density rho, the
 * parts of TotalFunctional.get_stress (total_functional.py:176-208) that the
 * evaluator owns: KEDF.stress (kedf/__init__.py:193-234) with TF
 * (kedf/tf.py:52-63), vW (kedf/vw.py:97-111) and WT (kedf/wt.py:75-106);
 * XC.stress with the built-in LDA (xc/__init__.py:80-95,
 * xc/semilocal_xc.py:343-346); Hartree.stress (hartree.py:51-90).
 * energies: the terms' energies that enter the diagonal (OFDFT_NE doubles, as
 * ofdft_eval_compute writes them), or NULL to compute them on rho first (the
 * reference uses the energies its functionals cached).  stress: OFDFT_NS x 9
 * doubles, zero for terms not configured.  The local pseudopotential and Ewald
 * terms come from ofdft_pseudo_stress and ofdft_ewald_stress.  With the
 * density-dependent (LWT) kernel it fails with OFDFT_EINVAL, as the reference's
 * KEDF.stress raises for 'LWT' (no stress engine, kedf/__init__.py:76-92). */
int ofdft_eval_stress(ofdft_eval* e, const void* rho, const double* energies, double* stress, ofdft_stream s);

/* Kernel table of the k_F-node term (lwt.py:535-566): its values at eta =
 * linspace(0, lwt_etamax, lwt_neta) (neta = lwt_neta), splined as the built-in
 * tables are.  Required with OFDFT_LWT_KERNEL_USER, e.g. the HC table, which the
 * reference integrates with scipy's odeint (kernel.py:460-478). */
int ofdft_eval_set_lwt_table(ofdft_eval* e, const double* table, int neta);

/* Stateful parts of the evaluator that persist across calls like the
 * reference's ke_kernel_saved (kedf/__init__.py:101-111): the k_F bound state
 * of the LWT rule (kedf/lwt.py:36-79).  get/set allow checkpoint and restore. */
int ofdft_eval_get_kfbounds(const ofdft_eval* e, double* kfmin, double* kfmax);
int ofdft_eval_set_kfbounds(ofdft_eval* e, double kfmin, double kfmax);
/* kernel time accounting of the last compute: nodes used, kernel launches */
int ofdft_eval_last_stats(const ofdft_eval* e, int* nsp, int* launches);

/* Per-kernel-class profiling with CUDA events recorded on the compute stream
 * around each launch (no counterpart in the reference, which times whole
 * calls with wall clocks in src/dftpy/time_data.py:94-122).  While enabled,
 * every compute accumulates, per class, the summed event time (ms), the
 * algorithmic bytes the launches must move, and the launch count.
 * ofdft_profile_class_name(i) names class i (NULL past the last class). */
int ofdft_eval_profile(ofdft_eval* e, int enable);
int ofdft_eval_profile_read(const ofdft_eval* e, int max_classes, double* ms, double* bytes, long long* launches,
                            int* nclasses);
const char* ofdft_profile_class_name(int i);

/* ------------------------------------------------- local pseudopotential
 * LocalPseudo (src/dftpy/functional/pseudo/__init__.py:74-452, :505-571).
 * Radial tables per species: v(q) on a uniform grid gp[0..npts-1] (gp[0]=0),
 * as read from a recpot file (recpot.py:11-42).  positions: nat x 3 Cartesian
 * (Bohr).  species: per-atom index into the tables. */
typedef struct ofdft_pseudo ofdft_pseudo;

int ofdft_pseudo_create(ofdft_grid* g, int nspecies, const int* npts, const double* const* gp,
                        const double* const* vp, int pme, int bspline_order, ofdft_pseudo** out);
void ofdft_pseudo_destroy(ofdft_pseudo* p);
int ofdft_pseudo_set_ions(ofdft_pseudo* p, int nat, const double* pos, const int* species);
/* v_loc(r) on the grid (LocalPseudo.local_PP, :237-246): PME (:437-452) or exact (:425-435) */
int ofdft_pseudo_vloc(ofdft_pseudo* p, void* vreal_out, ofdft_stream s);
/* LocalPseudo.forces (:260-270): PME (_ForcePME :523-571) or exact (_Force :505-521) */
int ofdft_pseudo_forces(ofdft_pseudo* p, const void* rho, double* forces, ofdft_stream s);
/* Gradient of E_PP = int v_loc rho dV with respect to every value of every
 * species' radial table vp (the v_loc(G) coefficients), by the adjoint of the
 * spline fit and of the structure-factor path; grad holds sum(npts) doubles,
 * species in order.  The reference has no counterpart (it offers no table
 * derivatives); the test pins it to finite differences of the oracle. */
int ofdft_pseudo_vloc_grad(ofdft_pseudo* p, const void* rho, double* grad, ofdft_stream s);
/* LocalPseudo.stress (:248-258): PME (_StressPME :573-611) or exact (_Stress
 * :479-503), with the radial derivative of each species' spline
 * (_PP_Derivative_One :454-460).  energy: E_PP = int v_loc rho dV, or NaN to
 * compute it here.  stress: 9 doubles (3 x 3, row-major). */
int ofdft_pseudo_stress(ofdft_pseudo* p, const void* rho, double energy, double* stress, ofdft_stream s);

/* ---------------------------------------------------------------- Ewald
 * ewald (src/dftpy/ewald.py:197-864): eta from Get_Best_eta (:256-278),
 * real-space erfc sum on a cell list, reciprocal part by PME (B-spline
 * order) or exact structure factors, and the G=0 / self corrections.
 * out_energy: [total, real, reciprocal, correction]; forces nat x 3 (may be NULL). */
int ofdft_ewald(ofdft_grid* g, int nat, const double* pos, const double* charges, double precision,
                int pme, int bspline_order, double* out_energy, double* forces, double* out_eta,
                ofdft_stream s);
/* ewald.stress (ewald.py:523-538): Stress_real (:609-662) plus Stress_rec_PME
 * (:915-968) or Stress_rec (:719-763), the G = 0 term included.  stress: 9
 * doubles (3 x 3, row-major); out_eta may be NULL. */
int ofdft_ewald_stress(ofdft_grid* g, int nat, const double* pos, const double* charges, double precision,
                       int pme, int bspline_order, double* stress, double* out_eta, ofdft_stream s);

/* ----------------------------------------------------------- optimiser
 * Optimization.optimize_rho (src/dftpy/optimization/optimization.py:283-525):
 * direct minimisation on phi = sqrt(rho) with the norm-conserving rotation
 * phi cos(theta) + p sin(theta), directions TN / LBFGS / CG-HS, and the
 * MINPACK-2 (More-Thuente) line search of scipy's line_search_wolfe1
 * (math_utils.py:37-52).  rho is overwritten with the optimised density. */
/* direction methods of Optimization.get_direction (optimization.py:179-203):
 * TN, L-BFGS, the conjugate-gradient betas of get_direction_CG
 * (math_utils.py:326-349: HS, PR with max(beta, 0), DY, CD, LS, FR; CD's beta is the
 * reference's pointwise field -(r*r)/sum(d r_prev)), GD (steepest descent with the
 * line search) and DIIS (the reference's damped fixed point: two steps of 0.1 per
 * iteration, optimization.py:327-333, :429-441, :471-485) */
enum { OFDFT_OPT_TN = 0, OFDFT_OPT_LBFGS = 1, OFDFT_OPT_CGHS = 2, OFDFT_OPT_CGPR = 3, OFDFT_OPT_CGDY = 4,
       OFDFT_OPT_CGCD = 5, OFDFT_OPT_CGLS = 6, OFDFT_OPT_CGFR = 7, OFDFT_OPT_GD = 8, OFDFT_OPT_DIIS = 9 };
typedef struct {
    int method, maxiter, maxfun, maxls, ncheck, maxcor;
    double econv, c1, c2, xtol, h0;
    int verbose;
    /* ofdft_optimize_batch only: 1 = every round of evaluations of the batch in one
     * persistent cooperative launch (ofdft_batch_eval), replayed as a CUDA graph,
     * when every system is eligible (else as with 0); the results then equal the
     * single solves to rounding instead of bit for bit.  0 (default): per-system
     * evaluations on worker streams, bit for bit the single solves. */
    int batch_persistent;
    /* Not in the reference (which stops on the energy test alone and searches on
     * the energy): pconv > 0 also stops once the residual norm dP = int r^2 dV
     * falls to pconv; ls_grad = 1 searches theta on the directional derivative
     * alone (doubling, then regula falsi to |phi'| <= c2 |phi'(0)|), for float32
     * stages whose energies carry round-off larger than the last decreases; it
     * has no sufficient-decrease test, so it is meant for a stage that starts
     * near the ground state (after an energy line search has stalled), not from
     * a uniform density.  Defaults 0 and 0. */
    double pconv;
    int ls_grad;
    /* Not in the reference (whose searches start at theta = 1): ls_start = 1
     * starts the line searches of L-BFGS and TN, from the second iteration on,
     * at the length of the search direction before its normalisation (the
     * quasi-Newton or Newton step along it) times the previous accepted step's
     * ratio to its direction's length, capped at the search's bound; 0
     * (default) keeps the reference's start (and twice the last accepted step
     * for ls_grad).  ofdft_optimize_batch applies it per system with the same
     * results as the single solves.  The same sizeof as without it: it fills
     * the padding after ls_grad. */
    int ls_start;
} ofdft_opt_options;
typedef struct {
    int converged;            /* 0 converged, 1 line search failed, 2 max steps (optimization.py:444-516) */
    int niter, nfev;
    double energy, mu, dP;
} ofdft_opt_result;

void ofdft_opt_default(ofdft_opt_options* o);
int ofdft_optimize(ofdft_eval* e, void* rho, const ofdft_opt_options* o, ofdft_opt_result* r,
                   ofdft_stream s);
/* The same, also writing the potential of the returned density (the one of the
 * last accepted evaluation, the reference's `self.functional`,
 * optimization.py:517-523) to v_out (device, grid precision; may be NULL), so
 * the caller needs no further evaluation. */
int ofdft_optimize_v(ofdft_eval* e, void* rho, const ofdft_opt_options* o, ofdft_opt_result* r, void* v_out,
                     ofdft_stream s);

/* Lockstep L-BFGS over n independent systems (n <= 128), each with its own
 * evaluator on its own grid (uneven grids allowed; one precision): the same
 * algorithm and result per system as ofdft_optimize, with every vector
 * operation launched once for the whole batch and one stream synchronisation
 * per round of scalars instead of one per system.  There is no counterpart
 * in the reference (which solves one system per call); it serves the
 * batched ground states of many small systems.  o->method must be L-BFGS;
 * econv (may be NULL: o->econv for all) gives each system its own energy
 * tolerance.  rho[i] is overwritten with system i's density, r[i] receives
 * its result, v_out[i] (v_out or its entries may be NULL) its final potential. */
int ofdft_optimize_batch(int n, ofdft_eval** evs, void** rho, const ofdft_opt_options* o, const double* econv,
                         ofdft_opt_result* r, void** v_out, ofdft_stream s);

/* ---- Wang-Govind-Carter nonlocal kinetic kernel with the two-body Fermi wave
 * vector xi = ((k_F(r)^gamma + k_F(r')^gamma)/2)^(1/gamma) (Phys. Rev. B 60,
 * 16350 (1999)), through its second-order Taylor expansion about the Fermi
 * wave vector of rho0, on the Wang-Teter kernel (kernel.py:325-334, lbda = x).
 * No counterpart in the reference.  rho0 <= 0: the mean density of each call
 * (kernel tables rebuilt when it moves by more than 1e-6).  compute writes the
 * nonlocal energy (Hartree) and, with OFDFT_CALC_V, its potential to v_out
 * (device, grid precision). */
typedef struct ofdft_wgc ofdft_wgc;
int ofdft_wgc_create(ofdft_grid* g, double alpha, double beta, double gamma, double x, double rho0,
                     ofdft_wgc** out);
int ofdft_wgc_compute(ofdft_wgc* w, const void* rho, void* v_out, unsigned calc, double* energy, ofdft_stream s);
void ofdft_wgc_destroy(ofdft_wgc* w);

/* ---- Persistent batched evaluation.  No counterpart in the reference, which
 * evaluates one system per call; it serves many small independent systems.
 * One cooperative launch evaluates E and V of every system of a batch (uneven
 * grids, one precision): the pre-pass, the forward and inverse transforms
 * (the library's own mixed-radix FFTs, axis lengths products of 2, 3 and 5 up
 * to 128), the Hartree and vW G-space factors and the post-pass of all
 * systems, stage by stage, with grid-wide barriers between stages.
 * Eligible evaluators use only TF, vW (no smoothing), LDA, Hartree and the
 * local pseudopotential; ofdft_batch_eval_eligible tells (1) or not (0).
 * Energies equal the evaluator's own to rounding (its transforms are cuFFT's);
 * repeated runs give the same bits. */
typedef struct ofdft_batch_eval ofdft_batch_eval;
int ofdft_batch_eval_eligible(ofdft_eval* e);
/* n (1..128) evaluators.  tune != 0 with rho and v_work (device fields of each
 * system, grid precision): a project autotuner times every candidate launch
 * shape (block 128/256 threads, 2/4/8 rows per row tile, 8/16/32 lines per
 * column tile) on this batch, overwriting v_work, and keeps the fastest for
 * every later batch of the same grids and precision in this process; otherwise
 * the kept shape, or block 256, 4 rows, 16 lines. */
int ofdft_batch_eval_create(int n, ofdft_eval** evs, int tune, void* const* rho, void* const* v_work,
                            ofdft_stream s, ofdft_batch_eval** out);
/* E and V of the systems with active[i] != 0 (active NULL: all): rho[i] in,
 * v_out[i] out (device, grid precision).  energies (host, n x OFDFT_NE, may be
 * NULL): filled for the active systems after the stream has been waited for;
 * with NULL the call returns once the work is enqueued.  Runs on one handle must
 * not overlap: the active mask and the energies live in the handle's pinned
 * buffers (wait for a run before starting the next). */
int ofdft_batch_eval_run(ofdft_batch_eval* b, void* const* rho, void* const* v_out, const unsigned char* active,
                         double* energies, ofdft_stream s);
/* the launch shape in use: threads per block, rows per row tile, lines per
 * column tile, blocks of the cooperative grid, and the tuned time per run (ms,
 * 0 when not tuned here) */
int ofdft_batch_eval_shape(const ofdft_batch_eval* b, int* block, int* rows, int* lines, int* grid,
                           double* tuned_ms);
/* a launch shape from a stored tuning table (block 128 or 256, rows 1..16,
 * lines 1..64); kept for later batches of the same grids */
int ofdft_batch_eval_set_shape(ofdft_batch_eval* b, int block, int rows, int lines);
void ofdft_batch_eval_destroy(ofdft_batch_eval* b);

/* The scalar MINPACK-2 line search on a host callback, exposed for testing
 * against scipy.optimize line_search_wolfe1 (scalar_search_wolfe1). */
typedef int (*ofdft_phi_fn)(double alpha, double* f, double* g, void* ctx);
int ofdft_linesearch(ofdft_phi_fn fn, void* ctx, double f0, double g0, double stp0, double c1, double c2,
                     double amax, double amin, double xtol, int maxiter, double* stp_out, double* f_out,
                     double* g_out, int* nfev);

/* The derivative-only line search of ls_grad on a host callback (no counterpart
 * in the reference; exposed for testing): *stp_out is NaN when it fails. */
int ofdft_linesearch_grad(ofdft_phi_fn fn, void* ctx, double g0, double stp0, double c2, double amax, int maxiter,
                          double* stp_out, double* f_out, double* g_out, int* nfev);

#ifdef __cplusplus
}
#endif
#endif /* OFDFT_H */
