"""Density files for restart and exchange (src/dftpy/formats/io.py:12-220) in
three of the reference's formats, written and read in code of our own:

  snpy  a sequence of numpy .npy records (formats/snpy.py:1-146): a
        description [1, 2, 3, 4(, 5)], then the cell (Bohr), the atomic
        numbers, the Cartesian positions (Bohr), the volumetric data (C order)
        and optional information;
  xsf   XCrySDen crystal files (formats/xsf.py): Angstrom, the data grid
        periodic (n + 1 points per axis) in Fortran order, densities in A^-3;
  qepp  Quantum ESPRESSO post-processing files (formats/qepp.py): Bohr,
        ibrav 0 (explicit cell, scaled by celldm(1)) or 1/2, data in Fortran
        order, potentials in Rydberg.

``read(fname, format=None, kind='all')`` returns (ions, data, info) on the
host, data a float64 (n0, n1, n2) array; ``read_density`` returns a
``DirectField``; ``write``/``write_density`` take a field (device or host).
Only unpolarised data (rank 1) is supported.
"""
import os

import numpy as np

from .constants import BOHR, HARTREE
from .ions import Ions

__all__ = ["read", "write", "read_density", "write_density", "read_potential", "write_potential",
           "guess_format"]

_SYMBOLS = ("X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br "
            "Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er "
            "Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md "
            "No Lr Rf Db Sg Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og").split()
_NUMBER = {s: i for i, s in enumerate(_SYMBOLS)}

_FORMATS = {"snpy": "snpy", "xsf": "xsf", "qepp": "qepp", "pp": "qepp"}


def guess_format(fname):
    """io.py:40-52: the extension names the format."""
    ext = os.path.splitext(fname)[1].lower().lstrip(".")
    if ext not in _FORMATS:
        raise AttributeError("%s format not support yet" % ext)
    return _FORMATS[ext]


def _host(data):
    if hasattr(data, "as_subclass"):
        import torch
        data = data.as_subclass(torch.Tensor).detach().double().cpu().numpy()
    data = np.asarray(data, dtype=np.float64)
    if data.ndim != 3:
        raise NotImplementedError("only unpolarised (rank 1) volumetric data is supported")
    return data


# ------------------------------------------------------------------- snpy
def _read_snpy(fname, kind):
    ions = data = info = None
    with open(fname, "rb") as fh:
        desc = np.load(fh)
        lattice = numbers = pos = None
        for key in desc:
            rec = np.load(fh)
            if key == 1:
                lattice = rec
            elif key == 2:
                numbers = rec
            elif key == 3:
                pos = rec
                ions = Ions(symbols=[_SYMBOLS[int(z)] for z in numbers], positions=pos, cell=lattice)
                if kind == "ions":
                    break
            elif key == 4:
                if rec.ndim != 3:
                    raise NotImplementedError("only unpolarised (rank 1) volumetric data is supported")
                data = np.asarray(rec, dtype=np.float64)
            elif key == 5:
                info = rec
    return ions, data, info, lattice


def _write_snpy(fname, ions, data, information):
    desc = np.arange(1, 6) if information is not None else np.arange(1, 5)
    with open(fname, "wb") as fh:
        np.save(fh, desc)
        np.save(fh, np.asarray(ions.cell, dtype=np.float64))
        np.save(fh, np.array([_NUMBER[s] for s in ions.symbols]))
        np.save(fh, np.asarray(ions.positions, dtype=np.float64))
        np.save(fh, data)
        if information is not None:
            np.save(fh, information)


# -------------------------------------------------------------------- xsf
def _xsf_lines(f):
    for line in f:
        line = line.strip()
        if line and not line.startswith("#"):
            yield line


def _read_xsf(fname, kind, data_type):
    with open(fname) as f:
        it = _xsf_lines(f)
        if next(it).upper() != "CRYSTAL":
            raise AttributeError("Only support crystal xsf.")
        line = next(it).upper()
        cell = None
        if line.startswith("PRIMVEC"):
            cell = np.array([[float(x) for x in next(it).split()] for _ in range(3)])
            line = next(it).upper()
        if line.startswith("CONVVEC"):
            for _ in range(3):
                next(it)
            line = next(it).upper()
        sym, pos = [], []
        if line.startswith("PRIMCOORD"):
            nat = int(next(it).split()[0])
            for _ in range(nat):
                w = next(it).split()
                s = w[0]
                sym.append(_SYMBOLS[int(s)] if s.isdigit() else s)
                pos.append([float(x) for x in w[1:4]])
        ions = Ions(symbols=sym, positions=np.array(pos).reshape(-1, 3), cell=cell, units="ase")
        if kind == "ions":
            return ions, None, None, None
        for line in it:
            if line.upper().startswith("BEGIN_DATAGRID_3D"):
                break
        else:
            raise AttributeError("!!!ERROR : XSF file have some problem")
        n = [int(x) for x in next(it).split()[:3]]
        next(it)  # origin
        span = np.array([[float(x) for x in next(it).split()] for _ in range(3)])
        vals = []
        need = n[0] * n[1] * n[2]
        for line in it:
            if line.upper().startswith("END"):
                break
            vals.extend(float(x) for x in line.split())
        arr = np.array(vals[:need]).reshape(n, order="F")
        data = np.ascontiguousarray(arr[: n[0] - 1, : n[1] - 1, : n[2] - 1]) * BOHR ** 3  # per A^3 -> per Bohr^3
        if data_type == "potential":
            data = data / HARTREE
        return ions, data, None, span / BOHR


def _fmt(v):
    return "%.15e" % v


def _write_xsf(fname, ions, data, lattice, data_type):
    cell = np.asarray(ions.cell) * BOHR
    pos = np.asarray(ions.positions) * BOHR
    vals = data / BOHR ** 3  # the reference scales potentials by 1/Bohr^3 too (xsf.py:229-233)
    if data_type == "potential":
        vals = vals * HARTREE
    per = np.pad(vals, ((0, 1), (0, 1), (0, 1)), mode="wrap").ravel(order="F")
    span = np.asarray(lattice) * BOHR
    with open(fname, "w") as f:
        f.write("# dftpy_gb300\nCRYSTAL\nPRIMVEC\n")
        for r in cell:
            f.write("  " + "  ".join(_fmt(x) for x in r) + "\n")
        f.write("PRIMCOORD\n  %d 1\n" % len(pos))
        for s, p in zip(ions.symbols, pos):
            f.write("  %s  %s\n" % (s, "  ".join(_fmt(x) for x in p)))
        f.write("BEGIN_BLOCK_DATAGRID_3D\n  3d_datagrid_%s\n  BEGIN_DATAGRID_3D#0\n" % data_type)
        f.write("  %d %d %d\n" % tuple(s + 1 for s in data.shape))
        f.write("  0.0 0.0 0.0\n")
        for r in span:
            f.write("  " + "  ".join(_fmt(x) for x in r) + "\n")
        for i in range(0, per.size, 5):
            f.write("  " + "  ".join(_fmt(x) for x in per[i:i + 5]) + "\n")
        f.write("  END_DATAGRID_3D\nEND_BLOCK_DATAGRID_3D\n")


# ------------------------------------------------------------------- qepp
def _celldm_at(ibrav, celldm):
    """Bravais lattices of the reference reader (qepp.py:124-134): ibrav 1 and 2 (columns)."""
    a = celldm[0]
    if ibrav == 1:
        return a * np.identity(3)
    if ibrav == 2:
        at = np.zeros((3, 3))
        at[:, 0] = 0.5 * a * np.array([-1.0, 0.0, 1.0])
        at[:, 1] = 0.5 * a * np.array([0.0, 1.0, 1.0])
        at[:, 2] = 0.5 * a * np.array([-1.0, 1.0, 0.0])
        return at
    raise NotImplementedError("celldm2at is only implemented for ibrav = 0 and ibrav = 1")


def _read_qepp(fname, kind, data_type):
    with open(fname) as f:
        title = f.readline()
        w = [int(x) for x in f.readline().split()]
        nrx, nat, ntyp = w[0:3], w[6], w[7]
        w = f.readline().split()
        ibrav, celldm = int(w[0]), np.array([float(x) for x in w[1:]])
        if ibrav == 0:
            at = np.array([[float(x) for x in f.readline().split()] for _ in range(3)]) * celldm[0]
        else:
            at = _celldm_at(ibrav, celldm)
        gcutm, dual, ecut, plot_num = (float(x) for x in f.readline().split())
        info = {"ibrav": ibrav, "celldm": celldm, "gcutm": gcutm, "dual": dual, "ecut": ecut,
                "plot_num": int(plot_num), "title": title}
        atm, zval = [], {}
        for _ in range(ntyp):
            w = f.readline().split()
            atm.append(w[1])
            zval[w[1]] = float(w[2])
        sym, tau = [], []
        for _ in range(nat):
            w = f.readline().split()
            tau.append([float(x) for x in w[1:4]])
            sym.append(atm[int(w[4]) - 1])
        tau = np.array(tau).reshape(-1, 3)
        if ibrav == 0:
            ions = Ions(symbols=sym, positions=tau * celldm[0], cell=at)
        else:
            ions = Ions(symbols=sym, scaled_positions=tau, cell=at)
        ions.set_charges(zval)
        if kind == "ions":
            return ions, None, info, at
        vals = np.array(f.read().split(), dtype=np.float64)
    data = np.ascontiguousarray(vals[: nrx[0] * nrx[1] * nrx[2]].reshape(nrx, order="F"))
    if data_type == "potential":
        data = data * 0.5  # Ry -> Ha
    return ions, data, info, at


def _write_qepp(fname, ions, data, data_type, information):
    info = {"gcutm": 1.0, "dual": 4.0, "ecut": 1.0, "ibrav": 0}
    if information:
        info.update(information)
    cell = np.asarray(ions.cell)
    celldm = np.zeros(6)
    celldm[0] = float(np.linalg.norm(cell[0]))
    uniq = sorted(set(ions.symbols))
    zval = {}
    try:
        zval = ions.zval
    except Exception:
        pass
    vals = data * 2.0 if data_type == "potential" else data  # Ha -> Ry
    flat = vals.ravel(order="F")
    n = data.shape
    with open(fname, "w") as f:
        f.write(str(info.get("title", "dftpy_gb300\n")).rstrip("\n") + "\n")
        f.write("  %d %d %d %d %d %d %d %d\n" % (n[0], n[1], n[2], n[0], n[1], n[2], len(ions.symbols), len(uniq)))
        f.write("  0 " + " ".join(_fmt(x) for x in celldm) + "\n")
        for r in cell / celldm[0]:
            f.write("  " + " ".join(_fmt(x) for x in r) + "\n")
        f.write("  %s %s %s %d\n" % (_fmt(info["gcutm"]), _fmt(info["dual"]), _fmt(info["ecut"]),
                                     info.get("plot_num", 1 if data_type == "potential" else 0)))
        for i, s in enumerate(uniq):
            f.write("  %d %s %s\n" % (i + 1, s, _fmt(float(zval.get(s, 0.0)))))
        tau = np.asarray(ions.positions) / celldm[0]
        for i, (s, t) in enumerate(zip(ions.symbols, tau)):
            f.write("  %d %s %d\n" % (i + 1, " ".join(_fmt(x) for x in t), uniq.index(s) + 1))
        for i in range(0, flat.size, 5):
            f.write(" ".join("%22.15e" % x for x in flat[i:i + 5]) + "\n")


# ------------------------------------------------------------------- API
def read(fname, format=None, kind="all", data_type="density"):
    """io.py:54-127 on the host: (ions, data, info) for kind 'all', ions for
    'ions', data for 'data'.  ``info`` carries the grid lattice (Bohr) under
    'lattice' and the qepp header values."""
    fmt = format or guess_format(fname)
    if fmt == "snpy":
        ions, data, info, lattice = _read_snpy(fname, kind)
    elif fmt == "xsf":
        ions, data, info, lattice = _read_xsf(fname, kind, data_type)
    elif fmt == "qepp":
        ions, data, info, lattice = _read_qepp(fname, kind, data_type)
    else:
        raise AttributeError("%s format not support yet" % fmt)
    if kind == "ions":
        return ions
    if kind == "data":
        return data
    info = dict(info or {}) if not isinstance(info, np.ndarray) else {"information": info}
    info["lattice"] = lattice if lattice is not None else (ions.cell if ions is not None else None)
    return ions, data, info


def write(fname, ions=None, data=None, information=None, format=None, data_type="density", lattice=None):
    """io.py:129-164: write ions and a field; the grid lattice defaults to the
    field's grid (else the ions' cell)."""
    if isinstance(data, Ions) and not isinstance(ions, Ions):
        ions, data = data, ions
    if lattice is None:
        g = getattr(data, "grid", None)
        lattice = np.asarray(g.lattice) if g is not None else np.asarray(ions.cell)
    arr = _host(data)
    fmt = format or guess_format(fname)
    if fmt == "snpy":
        _write_snpy(fname, ions, arr, information)
    elif fmt == "xsf":
        _write_xsf(fname, ions, arr, lattice, data_type)
    elif fmt == "qepp":
        _write_qepp(fname, ions, arr, data_type, information)
    else:
        raise AttributeError("%s format not support yet" % fmt)


def read_density(fname, format=None, dtype=None, **kwargs):
    """io.py:184-186: the density as a DirectField on its own grid (device)."""
    return _field(fname, format, dtype, "density")


def read_potential(fname, format=None, dtype=None, **kwargs):
    return _field(fname, format, dtype, "potential")


def _field(fname, format, dtype, data_type):
    import torch
    from .field import DirectField
    from .grid import DirectGrid
    ions, data, info = read(fname, format=format, kind="all", data_type=data_type)
    grid = DirectGrid(info["lattice"], data.shape)
    return DirectField(grid, data=data, dtype=dtype or torch.float64)


def write_density(fname, data=None, ions=None, format=None, **kwargs):
    return write(fname, ions=ions, data=data, format=format, data_type="density", **kwargs)


def write_potential(fname, data=None, ions=None, format=None, **kwargs):
    return write(fname, ions=ions, data=data, format=format, data_type="potential", **kwargs)
