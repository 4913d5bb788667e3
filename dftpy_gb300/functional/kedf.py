"""Kinetic energy density functionals on the accelerated path
(src/dftpy/functional/kedf/__init__.py:27-191): TF, vW, their combinations,
Wang-Teter (WT) and the density-dependent k_F-node kernel: LWT with the WT
kernel table (the WGC-style workload) and LMGP / LMGPA / LMGPG with the MGP
tables (kedf/lwt.py:571-578, kedf/kernel.py:267-322); and the GGA functionals
(kedf/gga.py), selected as the reference selects them (name 'GGA' with k_str,
or 'GGA_<functional>')."""
import copy

import numpy as np

from .. import _lib
from .abstract_functional import NativeFunctional
from .functional_output import FunctionalOutput, ZeroFunctional

__all__ = ["KEDF", "KEDFEngines"]

_BITS = {"HC-NL": _lib.KE_LWT, "REVHC-NL": _lib.KE_LWT, "GGA": _lib.KE_GGA, "TF": _lib.KE_TF, "VW": _lib.KE_VW, "WT-NL": _lib.KE_WT, "SM-NL": _lib.KE_WT, "FP-NL": _lib.KE_WT,
         "WTE-NL": _lib.KE_TF | _lib.KE_WT, "MGP-NL": _lib.KE_WT, "MGPA-NL": _lib.KE_WT, "MGPG-NL": _lib.KE_WT,
         "MGP0-NL": _lib.KE_WT, "LKT": _lib.KE_GGA | _lib.KE_VW, "DTTF": _lib.KE_DTTF, "LWT-NL": _lib.KE_LWT, "LMGP-NL": _lib.KE_LWT,
         "LMGPA-NL": _lib.KE_LWT, "LMGPG-NL": _lib.KE_LWT}
# kernel table of each k_F-node engine (lwt.py:571-578 fix kerneltype for the LMGP names)
_TABLE_OF = {"LMGP-NL": "MGP", "LMGPA-NL": "MGPA", "LMGPG-NL": "MGPG"}
_KERNELS = {"WT": _lib.LWT_KERNEL_WT, "MGP": _lib.LWT_KERNEL_MGP, "MGPA": _lib.LWT_KERNEL_MGPA,
            "MGPG": _lib.LWT_KERNEL_MGPG}

# name -> engines, as the reference's KEDFEngines table (kedf/__init__.py:27-69)
KEDFEngines = {
    "NONE": (),
    "TF": ("TF",),
    "VW": ("VW",),
    "X_TF_Y_VW": ("TF", "VW"),
    "XTFYVW": ("TF", "VW"),
    "TFVW": ("TF", "VW"),
    "WT": ("TF", "VW", "WT-NL"),
    "WT-NL": ("WT-NL",),
    "SM": ("TF", "VW", "SM-NL"),  # Smargiassi-Madden (sm.py): the WT engine with alpha = beta = 1/2
    "SM-NL": ("SM-NL",),
    "FP": ("TF", "VW", "FP-NL"),  # Perrot (fp.py): the WT engine with alpha = beta = 1
    "FP-NL": ("FP-NL",),
    "WTE": ("VW", "WTE-NL"),  # WTE (wte.py): E_TF exp(E_WT / E_TF)
    "WTE-NL": ("WTE-NL",),
    "MGP": ("TF", "VW", "MGP-NL"),  # density-independent MGP kernels (mgp.py)
    "MGPA": ("TF", "VW", "MGPA-NL"),
    "MGPG": ("TF", "VW", "MGPG-NL"),
    "MGP0": ("TF", "VW", "MGP0-NL"),
    "MGP-NL": ("MGP-NL",),
    "MGPA-NL": ("MGPA-NL",),
    "MGPG-NL": ("MGPG-NL",),
    "MGP0-NL": ("MGP0-NL",),
    "LWT": ("TF", "VW", "LWT-NL"),
    "LWT-NL": ("LWT-NL",),
    "LMGP": ("TF", "VW", "LMGP-NL"),
    "LMGPA": ("TF", "VW", "LMGPA-NL"),
    "LMGPG": ("TF", "VW", "LMGPG-NL"),
    "LMGP-NL": ("LMGP-NL",),
    "LMGPA-NL": ("LMGPA-NL",),
    "LMGPG-NL": ("LMGPG-NL",),
    "GGA": ("GGA",),
    "MGGA": ("GGA",),
    "LKT": ("LKT",),  # lkt.py: GGA 'LKT-VW' plus vW
    "DTTF": ("DTTF",),  # TTF - TF (tf.py:83-204), added to any name given a temperature
    "HC": ("TF", "VW", "HC-NL"),
    "REVHC": ("TF", "VW", "REVHC-NL"),
    "HC-NL": ("HC-NL",),
    "REVHC-NL": ("REVHC-NL",),
}

# HC and revHC (hc.py:333-439): their defaults, and the enhancement factor of k_F
_HC = {"HC-NL": {"functional": "HC", "params": None}, "REVHC-NL": {"functional": "PBE2", "params": [0.1, 0.45]}}


def _hc_factor(functional, params):
    """The GGA formula and parameters of F(s) in HC's k_F (hc.py:115-131):
    'HC' F = 1 + lambda s^2 (the TFVW formula, p = [1, 3/5 lambda TKF0^2]);
    'PBE2/3/4' of GGAFs (gga.py:936-968), F = 1 + b ss^2 / (1 + a ss^2) (+ ...),
    which is the PBE formula with p = [b / a, b, ...]."""
    f = str(functional).upper()
    tk = 6.18733545256027186194
    if f == "HC":
        lam = 0.0 if params is None else float(params[0])
        return _lib.GGA_TFVW, [1.0, 3.0 / 5.0 * lam * tk * tk]
    if f in ("PBE2", "PBE3", "PBE4"):
        p = list(GGA_FUNCTIONALS[f][1]) if params is None else list(params)
        n = {"PBE2": 2, "PBE3": 3, "PBE4": 4}[f]
        p = (p + list(GGA_FUNCTIONALS[f][1])[len(p):])[:n]
        return _lib.GGA_PBE, [p[1] / p[0]] + p[1:]
    raise NotImplementedError("HC with the %s enhancement factor is not supported (HC, PBE2-4 are)" % f)


_HC_TABLES = {}


def hc_kernel_table(eta, beta=2.0 / 3.0, x=1.0):
    """HCKernelTable (kernel.py:460-478): beta eta K' = -5/3 F(eta; x, 1) + (5 - 3 beta)
    beta K integrated with scipy's odeint from eta[-1], K(eta[-1]) = -8/3 / ((5 - 3 beta)
    beta), down to 0; K[0] = 0; times C_TF 8 (3 pi^2).  F is evaluated as the
    reference evaluates it on the float odeint passes: the closed form wherever it
    applies (no large-eta series)."""
    key = (float(beta), float(x), float(eta[-1]), len(eta))
    if key in _HC_TABLES:
        return _HC_TABLES[key]
    from scipy.integrate import odeint

    def lind(e, lbda, mu, tol=1e-10):
        tol2 = tol / 10
        if e > tol2 and abs(e - 1.0) > tol2:
            return 1.0 / (0.5 + 0.25 * (1.0 - e ** 2) * np.log((1.0 + e) / np.abs(1.0 - e)) / e) - 3.0 * mu * e ** 2 - lbda
        if e < tol:
            return 1.0 - lbda + e ** 2 * (1.0 / 3.0 - 3.0 * mu)
        return 2.0 - lbda - 3.0 * mu + 20.0 * (e - 1.0)

    def deriv(k, e):
        d = -5.0 / 3.0 * lind(e, x, 1) + (5.0 - 3.0 * beta) * beta * k
        if e > 1e-20:
            d /= beta * e
        return d

    sol = odeint(deriv, -8.0 / 3.0 / ((5.0 - 3.0 * beta) * beta), eta[::-1])
    k = sol.ravel()[::-1].copy()
    k[0] = 0.0
    k *= 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0) * 8.0 * 3.0 * np.pi ** 2
    _HC_TABLES[key] = k
    return k

# GGA_KEDF_list (gga.py:587-643): functional -> (formula, default parameters).  The
# reference looks names up upper-cased, so its mixed-case 'PW91k' key is unreachable.
_L = _lib
GGA_FUNCTIONALS = {
    "LKT-VW": (_L.GGA_LKTVW, [1.3]), "LKT": (_L.GGA_LKT, [1.3, 1.0]),
    "DK": (_L.GGA_DK, [0.95, 14.28111, -19.5762, -0.05, 9.99802, 2.96085]),
    "LLP": (_L.GGA_LLP, [0.0044188, 0.0253]), "LLP91": (_L.GGA_LLP, [0.0044188, 0.0253]),
    "OL1": (_L.GGA_OL, [0.00677, 0.0]), "OL": (_L.GGA_OL, [0.00677, 0.0]), "OL2": (_L.GGA_OL, [0.0887, 1.0]),
    "T92": (_L.GGA_THAK, [0.0055, 0.0253, 0.072]), "THAK": (_L.GGA_THAK, [0.0055, 0.0253, 0.072]),
    "B86A": (_L.GGA_B86A, [0.0039, 0.004]), "B86": (_L.GGA_B86A, [0.0039, 0.004]),
    "B86B": (_L.GGA_B86B, [0.00403, 0.007]),
    "DK87": (_L.GGA_DK87, [7.0 / 324.0 / (18.0 * np.pi ** 4) ** (1.0 / 3.0), 0.861504, 0.044286]),
    "PW86": (_L.GGA_PW86, [1.296, 14.0, 0.2]),
    "PW91O": (_L.GGA_PW91O, [0.093907, 0.26608, 0.0809615, 100.0, 76.320, 0.57767e-4]),
    "PW91": (_L.GGA_PW91, [0.19645, 0.2747, 0.1508, 100.0, 7.7956, 0.004]),
    "LG94": (_L.GGA_LG94, [(1e-8 + 0.1234) / 0.024974, 29.790, 22.417, 12.119, 1570.1, 55.944, 0.024974]),
    "E00": (_L.GGA_P92, [135.0, 28.0, 5.0, 3.0]), "P92": (_L.GGA_P92, [1.0, 88.3960, 16.3683, 88.2108]),
    "PBE2": (_L.GGA_PBE, [2.0309 / 0.2942, 2.0309]), "PBE3": (_L.GGA_PBE, [-3.7425 / 4.1355, -3.7425, 50.258]),
    "PBE4": (_L.GGA_PBE, [-7.2333 / 1.7107, -7.2333, 61.645, -93.683]), "P82": (_L.GGA_P82, [5.0 / 27.0]),
    "TW02": (_L.GGA_PBE, [0.8438, 0.2319]), "APBE": (_L.GGA_PBE, [0.804, 0.23889]),
    "APBEK": (_L.GGA_PBE, [0.804, 0.23889]), "REVAPBEK": (_L.GGA_PBE, [1.245, 0.23889]),
    "REVAPBE": (_L.GGA_PBE, [1.245, 0.23889]), "RPBE": (_L.GGA_PBE, [1.9632, 0.01979]),
    "VJKS00": (_L.GGA_VJKS00, [0.8944, 0.6511, 0.0431]),
    "LC94": (_L.GGA_PW91, [0.093907, 0.26608, 0.0809615, 100.0, 76.32, 0.000057767]),
    "VT84F": (_L.GGA_VT84F, [2.777028126, 2.777028126 - 40.0 / 27.0]),
    "TF": (_L.GGA_TFVW, [1.0, 0.0]), "VW": (_L.GGA_TFVW, [0.0, 1.0]), "X_TF_Y_VW": (_L.GGA_TFVW, [1.0, 1.0]),
    "TFVW": (_L.GGA_TFVW, [1.0, 1.0]), "STV": (_L.GGA_STV, [1.0, 1.0, 0.01, 1.0]),
    "PBE2M": (_L.GGA_PBE2M, [1.0, 0.2942, 2.0309]), "PG": (_L.GGA_PG, [0.75, 1.0]),
}

# MGGA_KEDF_list (gga.py:645-650): Laplacian-level functionals F(s, q)
MGGA_FUNCTIONALS = {
    "GE2": (_L.GGA_GE2, [1.0, 5.0 / 27.0, 20.0 / 9.0]),
    "GE4": (_L.GGA_GE4, [1.0, 5.0 / 27.0, 20.0 / 9.0, 8.0 / 81.0, -1.0 / 9.0, 8.0 / 243.0]),
    "PGSL": (_L.GGA_PGSL, [0.25, 40.0 / 27.0, 1.0]),
    "PGSLR": (_L.GGA_PGSLR, [0.40, 0.20, 0.25, 40.0 / 27.0, 1.0]),
}


# engines with a stress (KEDFEngines_Stress, kedf/__init__.py:76-92): slot in the
# stress and energy arrays of the native evaluator
_STRESS = {"TF": (_lib.S_TF, _lib.E_TF), "VW": (_lib.S_VW, _lib.E_VW), "WT-NL": (_lib.S_NL, _lib.E_NL),
           "SM-NL": (_lib.S_NL, _lib.E_NL), "FP-NL": (_lib.S_NL, _lib.E_NL), "WTE-NL": (_lib.S_NL, _lib.E_NL),
           "GGA": (_lib.S_GGA, _lib.E_GGA)}
_STRESS_NAMES = ("TF", "VW", "X_TF_Y_VW", "XTFYVW", "TFVW", "WT", "WT-NL", "SM", "SM-NL", "FP", "FP-NL", "WTE",
                 "WTE-NL", "GGA")
# MGP engines -> their fixed symmetrization (None: the symmetrization option)
_MGP = {"MGP-NL": None, "MGPA-NL": "Arithmetic", "MGPG-NL": "Geometric", "MGP0-NL": None}
# default exponents of the WT-engine variants (sm.py:14, fp.py:14); SMStress defaults to 1 (sm.py:18)
_WT_AB = {"SM-NL": 0.5, "FP-NL": 1.0}


class KEDF(NativeFunctional):
    """KEDF(name, **options) with the reference's option names: x, y, alpha, beta,
    rho0 (WT); nsp, delta, ratio, kdd, interp, etamax, neta, kfmin, kfmax, ldw (LWT)."""

    energy_slot = _lib.E_TOTAL
    out_name = "KEDF"

    def __init__(self, name="WT", kedf=None, **kwargs):
        self.type = "KEDF"
        self.name = (kedf or name).upper()
        kwargs = dict(kwargs)
        if self.name.startswith("GGA_"):  # kedf/__init__.py:134-137
            kwargs["k_str"] = self.name[4:]
            self.name = "GGA"
        if self.name.startswith("MGGA_"):  # kedf/__init__.py:138-142
            kwargs["k_str"] = self.name[5:]
            self.name = "MGGA"
        if self.name == "MGGA":
            kwargs["mgga"] = True
        if self.name not in KEDFEngines:
            raise NotImplementedError("KEDF %r is not on the accelerated path (have %s)" % (self.name,
                                                                                          sorted(KEDFEngines)))
        self.options = dict(kwargs)
        self.ke_kernel_saved = {"Kernel": None, "rho0": 0.0, "shape": None, "KernelTable": None, "etamax": None,
                                "KernelDeriv": None, "MGPKernelE": None, "kfmin": None, "kfmax": None}
        self.energies = {}
        self._check_options()

    def _check_options(self):
        o = self.options
        if str(o.get("kerneltype", "WT")).upper() not in _KERNELS:
            raise NotImplementedError("kernel tables WT, MGP, MGPA and MGPG are supported (got %r)"
                                      % o.get("kerneltype"))
        if o.get("symmetrization") not in (None, "None", "Arithmetic", "Geometric"):
            raise NotImplementedError("MGP symmetrization must be None, 'Arithmetic' or 'Geometric'")
        if o.get("lumpfactor") is not None and any(e in _TABLE_OF for e in self.engines()):
            raise NotImplementedError("lump factors of the LMGP family are not supported")
        if o.get("order", 3) != 3:
            raise NotImplementedError("kernel tables use cubic splines (order=3) only")
        if "GGA" in self.engines():
            k = o.get("k_str")
            if o.get("mgga"):  # gga.py:1226-1230
                if str(k or "LKT").upper() not in MGGA_FUNCTIONALS:
                    raise AttributeError("%s MGGA KEDF to be implemented" % str(k or "LKT").upper())
            elif k is not None and str(k).upper() not in GGA_FUNCTIONALS:
                raise AttributeError("%s GGA KEDF to be implemented" % str(k).upper())

    def engines(self, name=None):
        return KEDFEngines[(name or self.name).upper()]

    def configure(self, cfg, engines=None):
        o = self.options
        for e in (engines if engines is not None else self.engines()):
            cfg.kedf_terms |= _BITS[e]
        x = float(o.get("x", 1.0))
        cfg.tf_x = x
        cfg.vw_y = float(o.get("y", 1.0))
        engines = engines if engines is not None else self.engines()
        # Gaussian smoothing: of the vW Laplacian (vw.py:45-48) and of the GGA gradient (gga.py:1246-1250)
        sigma = o.get("sigma")
        sigma = 0.0 if sigma is None else float(sigma)
        cfg.vw_sigma = sigma if ("VW" in engines or "LKT" in engines) else 0.0
        cfg.wte = 1 if "WTE-NL" in engines else 0
        # a temperature adds the finite-temperature TF correction (kedf/__init__.py:155-156)
        t0, t = o.get("temperature0"), o.get("temperature")
        if t0 or t:
            cfg.kedf_terms |= _lib.KE_DTTF
            cfg.tf_temperature = float(t0 if t0 is not None else (t if t is not None else 1e-3))
            cfg.tf_temp_old = 1 if t0 is not None else 0
        mgp = next((e for e in engines if e in _MGP), None)
        if mgp:  # mgp.py:15-119: the kernel at rho0, its t integral and the lump correction
            sym = _MGP[mgp] or o.get("symmetrization")
            cfg.wt_kernel = {None: _lib.LWT_KERNEL_MGP, "None": _lib.LWT_KERNEL_MGP,
                             "Arithmetic": _lib.LWT_KERNEL_MGPA, "Geometric": _lib.LWT_KERNEL_MGPG}[sym]
            cfg.wt_maxpoints = int(o.get("maxpoint", 1000))
            cfg.wt_revke = 0 if mgp == "MGP0-NL" else 1
            # lumpfactor=None does not turn the lump correction off: KEDF drops
            # options set to None (kedf/__init__.py:144), so the default 0.2 applies
            lf = o.get("lumpfactor")
            if lf is None:
                lf = 0.2
            cfg.wt_lump_abc[2] = 1.0
            if isinstance(lf, (list, tuple)):
                cfg.wt_lump_abc[0] = float(lf[0])
                if len(lf) > 1:
                    cfg.wt_lump, cfg.wt_lump_abc[1] = 2, float(lf[1])
                else:
                    cfg.wt_lump = 1
                if len(lf) > 2:
                    cfg.wt_lump_abc[2] = float(lf[2])
            else:
                cfg.wt_lump, cfg.wt_lump_abc[0] = 1, float(lf)
        cfg.gga_sigma = sigma if ("GGA" in engines or "LKT" in engines) else 0.0
        hc = next((e for e in engines if e in _HC), None)
        wtv = next((_WT_AB[e] for e in engines if e in _WT_AB), None)
        a = float(o.get("alpha", 2.0 if hc else (wtv if wtv is not None else 5.0 / 6.0)))
        b = float(o.get("beta", 2.0 / 3.0 if hc else (wtv if wtv is not None else 5.0 / 6.0)))
        cfg.wt_alpha, cfg.wt_beta, cfg.wt_x = a, b, x
        rho0 = o.get("rho0")
        cfg.wt_rho0 = float(rho0) if rho0 else 0.0
        cfg.lwt_alpha, cfg.lwt_beta, cfg.lwt_x = a, b, x
        nsp, delta = o.get("nsp"), o.get("delta")
        cfg.lwt_nsp = int(nsp) if nsp is not None else 0
        cfg.lwt_delta = float(delta) if (nsp is None and delta is not None) else 0.0
        cfg.lwt_ratio = float(o.get("ratio", 1.15))
        cfg.lwt_kdd = int(o.get("kdd", 3))
        interp = str(o.get("interp", "hermite" if hc else "linear")).lower()
        if interp == "newton":
            interp = "linear"
        if interp not in ("linear", "hermite"):
            raise NotImplementedError("interp %r is not supported" % interp)
        cfg.lwt_interp = _lib.INTERP_HERMITE if interp == "hermite" else _lib.INTERP_LINEAR
        cfg.lwt_etamax = float(o.get("etamax", 50.0))
        cfg.lwt_neta = int(o.get("neta", 50000))
        cfg.lwt_kfmin = float("nan") if o.get("kfmin") is None else float(o["kfmin"])
        cfg.lwt_kfmax = float("nan") if o.get("kfmax") is None else float(o["kfmax"])
        ldw = o.get("ldw")
        cfg.lwt_ldw = 1.0 / 6.0 if ldw is None else float(ldw)
        cfg.lwt_max_batch = int(o.get("max_batch", 0))
        pipe = str(o.get("pipeline", "auto")).lower()
        pipes = {"auto": _lib.LWT_PIPE_AUTO, "cufft": _lib.LWT_PIPE_CUFFT, "fused": _lib.LWT_PIPE_FUSED,
                 "fused-split": _lib.LWT_PIPE_FUSED_SPLIT}
        if pipe not in pipes:
            raise ValueError("pipeline must be one of %s" % sorted(pipes))
        cfg.lwt_pipeline = pipes[pipe]
        # kernel table: fixed by the LMGP names, else the kerneltype option (lwt.py:535-548)
        engines = engines if engines is not None else self.engines()
        table = next((_TABLE_OF[e] for e in engines if e in _TABLE_OF), None)
        if table is None:
            table = str(o.get("kerneltype", "WT")).upper()
        if table == "MGP" and o.get("symmetrization") in ("Arithmetic", "Geometric"):
            table = "MGPA" if o.get("symmetrization") == "Arithmetic" else "MGPG"
        cfg.lwt_kernel = _KERNELS[table]
        cfg.lwt_maxpoints = int(o.get("maxpoints", 1000))
        if hc:  # HC / revHC: k_F from F(s), HC nodes and kernel, the table integrated on the host
            if interp != "hermite":
                raise NotImplementedError("HC is built with Hermite interpolation (its default) only")
            d = _HC[hc]
            formula, p = _hc_factor(o.get("functional", d["functional"]), o.get("params", d["params"]))
            cfg.lwt_family = _lib.LWT_FAMILY_HC
            cfg.lwt_kernel = _lib.LWT_KERNEL_USER
            cfg.gga_formula = formula
            cfg.gga_nparams = len(p)
            for i, v in enumerate(p):
                cfg.gga_params[i] = float(v)
        if "GGA" in engines or "LKT" in engines:  # gga.py:1212-1270: k_str's functional, default LKT
            name = "LKT-VW" if "LKT" in engines else str(o.get("k_str") or "LKT").upper()
            formula, p0 = (MGGA_FUNCTIONALS if o.get("mgga") else GGA_FUNCTIONALS)[name]
            params = o.get("params")
            p = list(p0)
            if params is not None:  # prefix replaced, extra values dropped (gga.py:1255-1265)
                params = [params] if isinstance(params, (int, float)) else list(params)
                p[:min(len(params), len(p))] = params[:len(p)]
            cfg.gga_formula = formula
            cfg.gga_nparams = len(p)
            for i, v in enumerate(p):
                cfg.gga_params[i] = float(v)
            rv = o.get("gga_remove_vw")
            cfg.gga_remove_vw = 0.0 if rv is None else (float(rv) if isinstance(rv, (int, float)) else 1.0)

    def prepare(self, ev, grid, dtype):
        s = self.ke_kernel_saved
        ev.set_kfbounds(s.get("kfmin"), s.get("kfmax"))
        if ev.cfg.lwt_family == _lib.LWT_FAMILY_HC and not getattr(ev, "lwt_table_set", False):
            c = ev.cfg
            eta = np.linspace(0, c.lwt_etamax, c.lwt_neta)
            ev.set_lwt_table(hc_kernel_table(eta, beta=c.lwt_beta, x=c.lwt_x))

    def finish(self, ev):
        kmin, kmax = ev.kfbounds()
        self.ke_kernel_saved["kfmin"] = kmin
        self.ke_kernel_saved["kfmax"] = kmax

    def compute(self, density, calcType={"E", "V"}, name=None, kedf=None, split=False, **kwargs):
        if kedf:
            name = kedf
        engines = self.engines(name)
        if not engines:
            return ZeroFunctional.compute(density, calcType=calcType)
        if not split:
            if name is None or name.upper() == self.name:
                return NativeFunctional.compute(self, density, calcType)
            sub = KEDF(name=name, **self.options)
            sub.ke_kernel_saved = self.ke_kernel_saved
            return NativeFunctional.compute(sub, density, calcType)
        out = {}
        o = self.options
        if o.get("temperature0") or o.get("temperature"):  # DTTF as its own part (kedf/__init__.py:155-156)
            engines = tuple(engines) + ("DTTF",)
        plain = {k: v for k, v in o.items() if k not in ("temperature", "temperature0")}
        for e in engines:
            sub = KEDF(name=e, **(o if e == "DTTF" else plain))
            sub.ke_kernel_saved = self.ke_kernel_saved
            r = NativeFunctional.compute(sub, density, calcType)
            r.name = e
            out[e] = r
            if "E" in calcType:
                self.energies[e] = r.energy
        return out

    def stress(self, density, name=None, kedf=None, split=False, **kwargs):
        """KEDF.stress (kedf/__init__.py:193-234): per engine, ThomasFermiStress
        (tf.py:52-63), vonWeizsackerStress (vw.py:97-111), WTStress (wt.py:75-106),
        with the energies the functional cached by a split compute (computed on
        this density when fewer than the engines are cached, as the reference does).
        Names without a stress engine (the LWT family among them) raise
        AttributeError, as the reference's name lookup does."""
        if kedf:
            name = kedf
        if name is None:
            name = self.name
        name = name.upper()
        if name not in _STRESS_NAMES:
            raise AttributeError("'{}' has not implemented.".format(name))
        if "GGA" in self.engines(name) and self.options.get("mgga"):
            raise AttributeError("Stress not support MGGA yet")
        engines = self.engines(name)
        if len(self.energies) < len(engines):
            self.compute(density, calcType={"E"}, name=name, split=True)
        E = np.zeros(_lib.NE)
        for e in engines:
            E[_STRESS[e][1]] = self.energies[e]
        opts = dict(self.options)
        if "SM-NL" in engines:  # SMStress takes alpha = beta = 1 unless given (sm.py:18-19)
            opts.setdefault("alpha", 1.0)
            opts.setdefault("beta", 1.0)
        sub = KEDF(name=name, **opts)
        sub.ke_kernel_saved = self.ke_kernel_saved
        S = sub._native_stress(density, E)
        out = {e: S[_STRESS[e][0]].copy() for e in engines}
        if split:
            return out
        return sum(out.values(), np.zeros((3, 3)))
