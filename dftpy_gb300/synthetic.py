"""Seeded synthetic systems for the OF-DFT hot path: crystal structures, the
analytic local pseudopotential and smooth trial densities.

No public data set is involved: every workload the tests and the benchmark use
is generated here from a seed.  Units are atomic (Bohr, Hartree).
"""
import numpy as np


def fcc_cell(a):
    """Conventional cubic fcc cell: lattice (rows) and the 4 Cartesian sites."""
    lattice = np.eye(3) * a
    frac = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
    return lattice, frac @ lattice


def bcc_cell(a):
    """Conventional cubic bcc cell: lattice (rows) and the 2 Cartesian sites."""
    lattice = np.eye(3) * a
    frac = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]])
    return lattice, frac @ lattice


def sc_cell(a):
    """Simple cubic cell: lattice (rows) and the single site."""
    return np.eye(3) * a, np.zeros((1, 3))


def supercell(lattice, positions, reps):
    """Repeat a cell reps=(r0, r1, r2) times; returns (lattice, positions)."""
    reps = np.asarray(reps, dtype=np.int64)
    shifts = np.array([[i, j, k] for i in range(reps[0]) for j in range(reps[1]) for k in range(reps[2])],
                      dtype=np.float64)
    pos = (positions[None, :, :] + (shifts @ lattice)[:, None, :]).reshape(-1, 3)
    return lattice * reps[:, None], pos


def fcc_supercell(a, reps, sigma=0.0, seed=0):
    """fcc Al-like supercell with seeded Gaussian displacements of width sigma (Bohr)."""
    lat, pos = fcc_cell(a)
    lat, pos = supercell(lat, pos, (reps, reps, reps) if np.isscalar(reps) else reps)
    if sigma > 0:
        rng = np.random.default_rng(seed)
        pos = pos + rng.normal(0.0, sigma, size=pos.shape)
    return lat, pos


def random_alloy(nat, density_e_per_bohr3, zvals, min_sep, seed=0, max_tries=2_000_000):
    """Uniform random positions with a minimum separation (rejection sampling) in a
    cubic box sized so that the valence electron density equals the target.
    ``zvals``: valence charge per species; species alternate 0,1,0,1... Returns
    (lattice, positions, species)."""
    species = np.arange(nat) % len(zvals)
    nelec = float(np.sum(np.asarray(zvals)[species]))
    L = (nelec / density_e_per_bohr3) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    pos = np.empty((0, 3))
    tries = 0
    while len(pos) < nat:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("random_alloy: could not place %d atoms" % nat)
        p = rng.uniform(0.0, L, size=3)
        if len(pos):
            d = pos - p
            d -= L * np.round(d / L)
            if np.min((d * d).sum(1)) < min_sep * min_sep:
                continue
        pos = np.vstack([pos, p])
    return np.eye(3) * L, pos, species


def analytic_vloc(Z, rc, A=15.0, npts=4096, gmax=40.0):
    """Radial local pseudopotential in G space on a uniform grid [0, gmax]:
    v(G) = -4 pi Z/G^2 exp(-G^2 rc^2/4) + A exp(-G^2 rc^2/4), with the finite
    G=0 limit A + pi Z rc^2 (so that the recpot zval rule recovers Z)."""
    g = np.linspace(0.0, gmax, npts)
    v = np.empty_like(g)
    e = np.exp(-g[1:] ** 2 * rc ** 2 / 4.0)
    v[1:] = -4.0 * np.pi * Z / g[1:] ** 2 * e + A * e
    v[0] = A + np.pi * Z * rc ** 2
    return g, v


def smooth_density(lattice, nr, nelec, seed=0, amp=0.3, kmax=3):
    """Positive, smooth, seeded trial density with a fixed electron count: rho0 *
    exp(s(r)) where s is a sum of low-|G| plane waves with random phases."""
    rng = np.random.default_rng(seed)
    nr = tuple(int(n) for n in nr)
    s = [np.arange(n) / n for n in nr]
    S = np.meshgrid(*s, indexing="ij")
    field = np.zeros(nr)
    for _ in range(12):
        k = rng.integers(-kmax, kmax + 1, size=3)
        ph = rng.uniform(0, 2 * np.pi)
        field += np.cos(2 * np.pi * (k[0] * S[0] + k[1] * S[1] + k[2] * S[2]) + ph)
    field *= amp / max(1e-12, np.abs(field).max())
    rho = np.exp(field)
    vol = abs(np.linalg.det(lattice))
    rho *= nelec / (rho.sum() * vol / rho.size)
    return rho


def atomic_density(lattice, nr, positions, zvals, width=1.2, floor=0.0):
    """Superposition of periodic Gaussians of charge zvals[a] at each site plus a
    floor; normalised to sum(zvals) electrons.  Used for vacuum-like trial
    densities where rho spans many orders of magnitude.  Orthorhombic cells use
    separable stencils truncated at 6 widths (exp(-18) relative); other cells
    sum over the whole grid per atom."""
    nr = tuple(int(n) for n in nr)
    lattice = np.asarray(lattice, dtype=np.float64)
    rho = np.full(nr, floor, dtype=np.float64)
    norm = (2 * np.pi * width ** 2) ** 1.5
    if np.allclose(lattice, np.diag(np.diag(lattice))):
        L = np.diag(lattice)
        cut = 6.0 * width
        for p, z in zip(positions, zvals):
            idx, val = [], []
            for d in range(3):
                h = L[d] / nr[d]
                c = p[d] / h
                w = min(int(np.ceil(cut / h)), nr[d] // 2)
                k = np.arange(int(np.floor(c)) - w, int(np.floor(c)) + w + 1)
                if len(k) > nr[d]:
                    k = k[:nr[d]]
                x = k * h - p[d]
                idx.append(np.mod(k, nr[d]))
                val.append(np.exp(-x * x / (2 * width ** 2)))
            rho[np.ix_(idx[0], idx[1], idx[2])] += (z / norm) * np.einsum("i,j,k->ijk", val[0], val[1], val[2])
    else:
        s = [np.arange(n) / n for n in nr]
        S = np.stack(np.meshgrid(*s, indexing="ij"), axis=-1)
        inv = np.linalg.inv(lattice)
        for p, z in zip(positions, zvals):
            f = S - (p @ inv)
            f -= np.round(f)
            r = f @ lattice
            rr = (r * r).sum(-1)
            rho += z * np.exp(-rr / (2 * width ** 2)) / norm
    vol = abs(np.linalg.det(lattice))
    rho *= float(np.sum(zvals)) / (rho.sum() * vol / rho.size)
    return rho


# (cell builder, repetitions) pairs whose supercells hold 4 to 108 atoms
_BATCH_SHAPES = [(fcc_cell, 1), (fcc_cell, 2), (fcc_cell, 3), (bcc_cell, 2), (bcc_cell, 3), (sc_cell, 2),
                 (sc_cell, 3), (sc_cell, 4)]
_BATCH_GRIDS = (48, 64, 72, 80, 96)


def batch_systems(count=64, seed=64, sigma=0.1, a_range=(7.3, 7.9)):
    """Independent systems of uneven size for batched ground states: fcc, bcc or
    sc cells repeated to 4-108 atoms, lattice constant uniform in a_range,
    seeded Gaussian displacements of width sigma, grids drawn from
    {48, 64, 72, 80, 96}^3.  Returns a list of dicts (lattice, positions, nr, kind)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        build, reps = _BATCH_SHAPES[int(rng.integers(len(_BATCH_SHAPES)))]
        a = float(rng.uniform(*a_range))
        lat, pos = build(a)
        lat, pos = supercell(lat, pos, (reps, reps, reps))
        pos = pos + rng.normal(0.0, sigma, size=pos.shape)
        n = int(_BATCH_GRIDS[int(rng.integers(len(_BATCH_GRIDS)))])
        out.append({"lattice": lat, "positions": pos, "nr": (n, n, n),
                    "kind": "%s %dx%dx%d" % (build.__name__.replace("_cell", ""), reps, reps, reps)})
    return out
