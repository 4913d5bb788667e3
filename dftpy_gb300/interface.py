"""Config-driven density optimisation (src/dftpy/interface.py:150-229,
OptimizeDensityConf) on the device backend.

``config`` is the reference's nested configuration dictionary; the sections
this path reads are OPT, MIX, JOB, MATH, DENSITY and OUTPUT, with the
reference's defaults (src/dftpy/config/configentries.json) for any key left
out.  With ``config['OPT']['algorithm'] == 'OESCF'`` the optimisation runs as
OE-SCF with the embedding evaluator ``evaluator_emb`` and the configured mixer.
"""
import copy

import numpy as np

from .api import evaluator2results
from .field import DirectField
from .grid import DirectGrid
from .utils import field2distrib
from .constants import HARTREE
from .mixer import Mixer
from .optimization import OESCF, Optimization

__all__ = ["OptimizeDensityConf", "default_config"]

# the reference's defaults of the sections OptimizeDensityConf reads
_DEFAULTS = {
    "OPT": {"method": "CG-HS", "algorithm": "EMM", "vector": "Orthogonalization", "c1": 1e-4, "c2": 0.2,
            "maxls": 10, "econv": 1e-6, "maxfun": 50, "maxiter": 100, "xtol": 1e-12, "h0": 1},
    "MIX": {"scheme": "pulay", "predtype": "kerker", "predcoef": [1.0, 1.0, 1.0], "predecut": None, "maxm": 7,
            "coef": 0.7, "delay": 2, "restarted": False, "kf": "auto"},
    "JOB": {"task": "Optdensity", "calctype": "Energy"},
    "MATH": {"linearii": True, "linearie": True, "twostep": False, "multistep": 1, "reuse": True},
    "DENSITY": {"densityoutput": None},
    "OUTPUT": {"electrostatic_potential": None, "stress": True},
    "GRID": {"gfull": False},
}


def default_config():
    """A fresh copy of the defaults of the sections OptimizeDensityConf reads."""
    return copy.deepcopy(_DEFAULTS)


def _merged(config):
    cfg = default_config()
    for sec, vals in (config or {}).items():
        if isinstance(vals, dict):
            cfg.setdefault(sec, {}).update(vals)
        else:
            cfg[sec] = vals
    return cfg


def OptimizeDensityConf(config, ions=None, rho=None, E_v_Evaluator=None, nr2=None, evaluator_emb=None, **kwargs):
    """interface.py:150-229: optimise the density as ``config`` says (OE-SCF or
    a direct optimisation), then evaluate what JOB.calctype asks for and return
    the results dictionary of evaluator2results."""
    config = _merged(config)
    rho_ini = rho
    lscf = config["OPT"]["algorithm"] == "OESCF"
    mix_kwargs = dict(config["MIX"])
    if mix_kwargs.get("predecut"):
        mix_kwargs["predecut"] *= 1.0 / HARTREE  # eV -> Hartree
    mixer = Mixer(nspin=1, **mix_kwargs)
    if "Optdensity" in config["JOB"]["task"]:
        optimization_options = dict(config["OPT"])
        optimization_options["econv"] *= ions.nat
        if lscf:
            optimization_options["algorithm"] = "EMM"
            if evaluator_emb is None:
                raise AttributeError("OE-SCF needs the embedding evaluator (evaluator_emb)")
        opt = Optimization(EnergyEvaluator=E_v_Evaluator, optimization_options=optimization_options,
                           optimization_method=config["OPT"]["method"])
        if lscf:
            opt = OESCF(optimization=opt, evaluator_emb=evaluator_emb, mixer=mixer)
        rho = opt.optimize_rho(guess_rho=rho_ini)
        # further steps on denser grids (interface.py:183-205)
        grid = rho_ini.grid
        nr = np.array(grid.nrR, dtype=int)
        charge_total = ions.get_ncharges()
        for istep in range(2, config["MATH"]["multistep"] + 1):
            if istep == config["MATH"]["multistep"]:
                if nr2 is None:
                    nr2 = nr * 2
                nr = np.array(nr2, dtype=int)
            else:
                nr = nr * 2
            grid2 = DirectGrid(lattice=grid.lattice, nr=nr, full=config["GRID"]["gfull"])
            rho_ini = DirectField(grid2, dtype=rho.dtype)
            field2distrib(rho, rho_ini, root=0)
            rho_ini = rho_ini * (charge_total / float(rho_ini.integral()))
            pseudo = getattr(E_v_Evaluator, "PSEUDO", None)
            if pseudo is not None:
                pseudo.restart(full=False, ions=pseudo.ions, grid=grid2)
            rho = opt.optimize_rho(guess_rho=rho_ini)
    if lscf:
        E_v_Evaluator.UpdateFunctional(newFuncDict=evaluator_emb.funcDict)
    calcType = set()
    ct = config["JOB"]["calctype"]
    if "Both" in ct:
        calcType.update({"E", "V"})
    if "Potential" in ct:
        calcType.add("V")
    if "Energy" in ct:
        calcType.add("E")
    if "Force" in ct:
        calcType.add("F")
    if "Stress" in ct:
        calcType.add("S")
    if config["DENSITY"]["densityoutput"]:
        from .formats import write_density
        write_density(config["DENSITY"]["densityoutput"], data=rho, ions=ions)
    if config["OUTPUT"]["electrostatic_potential"]:
        from .formats import write_density
        from .properties import get_electrostatic_potential
        write_density(config["OUTPUT"]["electrostatic_potential"], data=get_electrostatic_potential(rho, E_v_Evaluator),
                      ions=ions)
    results = evaluator2results(E_v_Evaluator, rho=rho, calcType=calcType, ions=ions, **kwargs)
    if lscf:
        E_v_Evaluator.UpdateFunctional(keysToRemove=evaluator_emb.funcDict)
    return results
