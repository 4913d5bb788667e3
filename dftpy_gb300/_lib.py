"""ctypes binding of the in-tree C-ABI library (include/ofdft.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
when ``libofdft.so`` is missing and cannot be built.
"""
import ctypes as C
import os
import threading

from . import _build

_LOCK = threading.Lock()
_LIB = None

OK, EINVAL, ECUDA, ECUFFT, ENOMEM, ESTATE = range(6)
F64, F32 = 0, 1
CALC_E, CALC_V = 1, 2
E_TF, E_VW, E_NL, E_XC, E_H, E_PP, E_II, E_TOTAL, E_NELEC, E_GGA, E_EXT, E_DTTF, NE = range(13)
S_TF, S_VW, S_NL, S_XC, S_H, S_GGA, NS = range(7)
KE_TF, KE_VW, KE_WT, KE_LWT, KE_GGA, KE_DTTF = 1, 2, 4, 8, 16, 32
(GGA_LKT, GGA_LKTVW, GGA_DK, GGA_LLP, GGA_OL, GGA_THAK, GGA_B86A, GGA_B86B, GGA_DK87, GGA_PW86, GGA_PW91O, GGA_PW91,
 GGA_LG94, GGA_P92, GGA_PBE, GGA_P82, GGA_VJKS00, GGA_VT84F, GGA_TFVW, GGA_STV, GGA_PBE2M, GGA_PG, GGA_GE2, GGA_GE4, GGA_PGSL, GGA_PGSLR) = range(26)
INTERP_LINEAR, INTERP_HERMITE = 0, 1
LWT_PIPE_AUTO, LWT_PIPE_CUFFT, LWT_PIPE_FUSED, LWT_PIPE_FUSED_SPLIT = 0, 1, 2, 3
LWT_KERNEL_WT, LWT_KERNEL_MGP, LWT_KERNEL_MGPA, LWT_KERNEL_MGPG, LWT_KERNEL_USER = 0, 1, 2, 3, 4
LWT_FAMILY_LWT, LWT_FAMILY_HC = 0, 1
OPT_TN, OPT_LBFGS, OPT_CGHS, OPT_CGPR, OPT_CGDY, OPT_CGCD, OPT_CGLS, OPT_CGFR, OPT_GD, OPT_DIIS = range(10)
PRED_NONE, PRED_KERKER, PRED_INVERSE_KERKER, PRED_RESTA = 0, 1, 2, 3
MIX_MAXM = 8


class OfdftError(RuntimeError):
    """An error status returned by the C ABI."""


class Config(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint),
        ("kedf_terms", C.c_int),
        ("tf_x", C.c_double), ("vw_y", C.c_double),
        ("wt_alpha", C.c_double), ("wt_beta", C.c_double), ("wt_x", C.c_double), ("wt_rho0", C.c_double),
        ("lwt_alpha", C.c_double), ("lwt_beta", C.c_double), ("lwt_x", C.c_double),
        ("lwt_nsp", C.c_int), ("lwt_delta", C.c_double), ("lwt_ratio", C.c_double),
        ("lwt_kdd", C.c_int), ("lwt_interp", C.c_int), ("lwt_etamax", C.c_double), ("lwt_neta", C.c_int),
        ("lwt_kfmin", C.c_double), ("lwt_kfmax", C.c_double), ("lwt_ldw", C.c_double), ("lwt_max_batch", C.c_int),
        ("xc_lda", C.c_int), ("hartree", C.c_int), ("pseudo", C.c_int), ("ewald_energy", C.c_double),
        ("lwt_pipeline", C.c_int), ("lwt_kernel", C.c_int), ("lwt_maxpoints", C.c_int),
        ("gga_formula", C.c_int), ("gga_nparams", C.c_int), ("gga_params", C.c_double * 8),
        ("gga_remove_vw", C.c_double), ("lwt_family", C.c_int), ("external", C.c_int),
        ("vw_sigma", C.c_double), ("gga_sigma", C.c_double), ("wte", C.c_int),
        ("wt_kernel", C.c_int), ("wt_maxpoints", C.c_int), ("wt_lump", C.c_int), ("wt_lump_abc", C.c_double * 3),
        ("wt_revke", C.c_int), ("tf_temperature", C.c_double), ("tf_temp_old", C.c_int),
    ]


class OptOptions(C.Structure):
    _fields_ = [
        ("method", C.c_int), ("maxiter", C.c_int), ("maxfun", C.c_int), ("maxls", C.c_int), ("ncheck", C.c_int),
        ("maxcor", C.c_int), ("econv", C.c_double), ("c1", C.c_double), ("c2", C.c_double), ("xtol", C.c_double),
        ("h0", C.c_double), ("verbose", C.c_int), ("batch_persistent", C.c_int),
        ("pconv", C.c_double), ("ls_grad", C.c_int), ("ls_start", C.c_int),
    ]


class OptResult(C.Structure):
    _fields_ = [("converged", C.c_int), ("niter", C.c_int), ("nfev", C.c_int), ("energy", C.c_double),
                ("mu", C.c_double), ("dP", C.c_double)]


class MixArgs(C.Structure):
    _fields_ = [
        ("predtype", C.c_int), ("predcoef", C.c_double * 3), ("cutoff", C.c_int), ("predecut", C.c_double),
        ("coef", C.c_double), ("mask_coef", C.c_double), ("resw", C.c_double), ("ns", C.c_int),
        ("dn", C.c_void_p * MIX_MAXM), ("dr", C.c_void_p * MIX_MAXM), ("x", C.c_double * MIX_MAXM),
    ]


PHI_FN = C.CFUNCTYPE(C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)

_P = C.c_void_p
_D = C.c_double
_I = C.c_int
_PD = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int)

_SIGS = {
    "ofdft_last_error": (C.c_char_p, []),
    "ofdft_version": (C.c_char_p, []),
    "ofdft_grid_create": (_I, [_PI, _PD, _I, C.POINTER(_P)]),
    "ofdft_grid_destroy": (None, [_P]),
    "ofdft_grid_info": (_I, [_P, _PI, _PD, _PD, _PI]),
    "ofdft_fft": (_I, [_P, _P, _P, _P]),
    "ofdft_ifft": (_I, [_P, _P, _P, _P]),
    "ofdft_grid_map": (_I, [_P, _P, _P, _P, _D, _P]),
    "ofdft_dot": (_I, [_P, _P, _P, _PD, _P]),
    "ofdft_dot3": (_I, [_P, _P, _P, _P, _PD, _P]),
    "ofdft_dot_noalloc": (_I, [_P, _P, C.c_longlong, _I, _P, _P]),
    "ofdft_config_size": (C.c_size_t, []),
    "ofdft_config_init": (_I, [C.POINTER(Config), C.c_size_t]),
    "ofdft_config_default": (None, [C.POINTER(Config)]),
    "ofdft_eval_create": (_I, [_P, C.POINTER(Config), C.POINTER(_P)]),
    "ofdft_eval_destroy": (None, [_P]),
    "ofdft_eval_set_vloc": (_I, [_P, _P, _P]),
    "ofdft_eval_set_ewald": (_I, [_P, _D]),
    "ofdft_eval_set_external": (_I, [_P, _P, _P]),
    "ofdft_eval_compute": (_I, [_P, _P, _P, C.c_uint, _PD, _P]),
    "ofdft_eval_stress": (_I, [_P, _P, _PD, _PD, _P]),
    "ofdft_eval_set_lwt_table": (_I, [_P, _PD, _I]),
    "ofdft_eval_get_kfbounds": (_I, [_P, _PD, _PD]),
    "ofdft_eval_set_kfbounds": (_I, [_P, _D, _D]),
    "ofdft_eval_last_stats": (_I, [_P, _PI, _PI]),
    "ofdft_eval_profile": (_I, [_P, _I]),
    "ofdft_eval_profile_read": (_I, [_P, _I, _PD, _PD, C.POINTER(C.c_longlong), _PI]),
    "ofdft_profile_class_name": (C.c_char_p, [_I]),
    "ofdft_pseudo_create": (_I, [_P, _I, _PI, C.POINTER(_PD), C.POINTER(_PD), _I, _I, C.POINTER(_P)]),
    "ofdft_pseudo_destroy": (None, [_P]),
    "ofdft_pseudo_set_ions": (_I, [_P, _I, _PD, _PI]),
    "ofdft_pseudo_vloc": (_I, [_P, _P, _P]),
    "ofdft_pseudo_forces": (_I, [_P, _P, _PD, _P]),
    "ofdft_pseudo_stress": (_I, [_P, _P, _D, _PD, _P]),
    "ofdft_pseudo_vloc_grad": (_I, [_P, _P, _PD, _P]),
    "ofdft_ewald": (_I, [_P, _I, _PD, _PD, _D, _I, _I, _PD, _PD, _PD, _P]),
    "ofdft_ewald_stress": (_I, [_P, _I, _PD, _PD, _D, _I, _I, _PD, _PD, _P]),
    "ofdft_opt_default": (None, [C.POINTER(OptOptions)]),
    "ofdft_optimize": (_I, [_P, _P, C.POINTER(OptOptions), C.POINTER(OptResult), _P]),
    "ofdft_optimize_v": (_I, [_P, _P, C.POINTER(OptOptions), C.POINTER(OptResult), _P, _P]),
    "ofdft_optimize_batch": (_I, [_I, C.POINTER(_P), C.POINTER(_P), C.POINTER(OptOptions), C.POINTER(C.c_double),
                                  C.POINTER(OptResult), C.POINTER(_P), _P]),
    "ofdft_wgc_create": (_I, [_P, _D, _D, _D, _D, _D, C.POINTER(_P)]),
    "ofdft_wgc_compute": (_I, [_P, _P, _P, C.c_uint, _PD, _P]),
    "ofdft_wgc_destroy": (None, [_P]),
    "ofdft_batch_eval_eligible": (_I, [_P]),
    "ofdft_batch_eval_create": (_I, [_I, C.POINTER(_P), _I, C.POINTER(_P), C.POINTER(_P), _P, C.POINTER(_P)]),
    "ofdft_batch_eval_run": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(C.c_ubyte), _PD, _P]),
    "ofdft_batch_eval_shape": (_I, [_P, _PI, _PI, _PI, _PI, _PD]),
    "ofdft_batch_eval_set_shape": (_I, [_P, _I, _I, _I]),
    "ofdft_batch_eval_destroy": (None, [_P]),
    "ofdft_mix_history": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _P]),
    "ofdft_mix_gram": (_I, [_P, C.POINTER(_P), _I, _PD, _P]),
    "ofdft_mix_density": (_I, [_P, _P, _P, C.POINTER(MixArgs), _P, _P]),
    "ofdft_linesearch": (_I, [PHI_FN, _P, _D, _D, _D, _D, _D, _D, _D, _D, _I, _PD, _PD, _PD, _PI]),
    "ofdft_linesearch_grad": (_I, [PHI_FN, _P, _D, _D, _D, _D, _I, _PD, _PD, _PD, _PI]),
}


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libofdft.so (building it with nvcc first if needed)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if build_if_missing:
            try:
                path = _build.build()
            except Exception as exc:  # surface the real reason
                if not os.path.exists(path):
                    raise OfdftError("libofdft.so is missing and could not be built: %s" % exc) from exc
        if not os.path.exists(path):
            raise OfdftError("libofdft.so not found at %s; run __graft_entry__.build()" % path)
        lib = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.ofdft_config_size() != C.sizeof(Config):
            raise OfdftError("the ctypes mirror of ofdft_config has %d bytes, the library's %d: update "
                             "dftpy_gb300/_lib.py from include/ofdft.h" % (C.sizeof(Config), lib.ofdft_config_size()))
        _LIB = lib
        return lib


def check(rc):
    if rc != OK:
        msg = load().ofdft_last_error().decode(errors="replace")
        raise OfdftError("ofdft error %d: %s" % (rc, msg))


def exported_symbols():
    return list(_SIGS)


def dptr(arr):
    """Pointer to a contiguous float64 numpy array."""
    return arr.ctypes.data_as(_PD)
