"""Seeded input generators for the parity tests and the benchmark.

They restate the reference's test generators (test/test_utils.jl:28-52,
297-310) and the workload shapes of the benchmark configurations.  The
reference's RNG is unseeded; here every generator takes a seed and uses
numpy's PCG64, whose stream is the same on every platform.
"""
from __future__ import annotations

import numpy as np

ALL_PBC = [
    (True, True, True),
    (False, False, False),
    (True, False, False),
    (False, True, False),
    (False, False, True),
    (True, True, False),
    (True, False, True),
    (False, True, True),
]  # test_utils.jl:41-52


def rand_config(N, density=0.05, seed=0):
    """Uniform cubic box (test_utils.jl:28-34): returns X, cell, L."""
    rng = np.random.default_rng(seed)
    L = (N / density) ** (1.0 / 3.0)
    X = rng.random((N, 3)) * L
    return X, np.diag([L, L, L]), L


def corner_clump(N, cutoff, per_octant=28, density=0.05, seed=0):
    """A uniform cubic box whose 8 cells around one interior corner of the
    cell grid (floor(L / cutoff) cells per axis) hold only a clump of
    8 * per_octant atoms within 0.9 A of that corner, per_octant in each cell:
    the clump's atoms have more than 8 * per_octant - 1 pairs while no cell
    holds more than max(per_octant, background) atoms.  Returns X, cell, L."""
    X, C, L = rand_config(N, density, seed)
    ns = int(np.floor(L / cutoff))
    w = L / ns
    corner = np.full(3, (ns // 2) * w)
    X = X[np.any(np.abs(X - corner) >= w, axis=1)]
    rng = np.random.default_rng(seed + 1)
    signs = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)], dtype=float)
    clump = corner + np.repeat(signs, per_octant, axis=0) * rng.uniform(0.05, 0.9 / np.sqrt(3), (8 * per_octant, 3))
    return np.concatenate([X, clump]), C, L


def triclinic_cell():
    """rand_non_cubic_cell (test_utils.jl:297-299); rows are lattice vectors."""
    return np.array([[10.0, 2.0, 1.0], [0.0, 9.0, 1.5], [0.0, 0.0, 8.0]])


def rand_config_triclinic(N, cell=None, seed=0):
    """test_utils.jl:306-310: X = cell' * rand."""
    cell = triclinic_cell() if cell is None else np.asarray(cell, dtype=np.float64)
    rng = np.random.default_rng(seed)
    return rng.random((N, 3)) @ cell, cell


def fcc_cubic(a, reps):
    """Cubic FCC supercell (conventional basis), atoms in [0, L)."""
    basis = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    g = np.stack(np.meshgrid(*[np.arange(r) for r in reps], indexing="ij"), -1).reshape(-1, 3)
    X = ((g[:, None, :] + basis[None, :, :]).reshape(-1, 3)) * a
    return X, np.diag(np.array(reps, dtype=np.float64) * a)


def fcc_sheared(n=20, a=3.61, sigma=0.05, vacuum=10.0, seed=0):
    """FCC a=3.61, n^3 conventional cells, Gaussian noise, cell sheared with
    h_xy = 0.1 L, h_xz = 0.05 L, 10 A of vacuum along z; pbc = (T, T, F)."""
    rng = np.random.default_rng(seed)
    L = n * a
    basis = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    g = np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3)
    frac = ((g[:, None, :] + basis[None, :, :]).reshape(-1, 3)) / n
    occupied = np.array([[L, 0, 0], [0.1 * L, L, 0], [0.05 * L, 0, L]])
    X = frac @ occupied + rng.normal(0.0, sigma, size=(frac.shape[0], 3))
    cell = np.array([[L, 0, 0], [0.1 * L, L, 0], [0.05 * L, 0, L + vacuum]])
    return X, cell, (True, True, False)


def diamond_primitive(a=5.43):
    """2-atom diamond primitive cell, basis (0,0,0) and (1/4,1/4,1/4)."""
    cell = a / 2 * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])
    X = np.array([[0.0, 0.0, 0.0], [0.25, 0.25, 0.25]]) @ cell
    return X, cell


def uniform_system(N, density=0.05, seed=0):
    """Large-system workload: N atoms uniform in a cubic pbc box."""
    return rand_config(N, density, seed)


def batch_systems(nsys, seed=0, nmin=8, nmax=4096):
    """Many small systems: N log-uniform in [nmin, nmax], triclinic cells with
    density U[0.03, 0.10] and off-diagonals U(+-0.15 diag), pbc per axis with
    probability 0.8, cutoff U[3, 6].  Returns [(X, cell, cutoff, pbc), ...]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nsys):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1))))
        n = min(max(n, nmin), nmax)
        rho = rng.uniform(0.03, 0.10)
        L = (n / rho) ** (1.0 / 3.0)
        cell = np.diag([L, L, L]) * rng.uniform(0.85, 1.15, size=3)
        for r in range(3):
            for c in range(3):
                if r != c:
                    cell[r, c] = rng.uniform(-0.15, 0.15) * cell[r, r]
        X = rng.random((n, 3)) @ cell
        pbc = tuple(bool(b) for b in rng.random(3) < 0.8)
        rc = rng.uniform(3.0, 6.0)
        out.append((X, cell, rc, pbc))
    return out
