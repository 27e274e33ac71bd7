"""Seeded synthetic atomic structures used by the tests and the benchmark.

MatPL measures nothing on public data for this path; the workloads here are synthetic
stand-ins with the shapes and value distributions of the benchmark configurations:

* ``fcc(...)``            — an FCC crystal (e.g. Cu, a = 3.615 A) with Gaussian displacements;
* ``random_packed(...)``  — random sequential insertion at a given number density with a
                            minimum pair distance (cell-list rejection), multi-element.

Every structure is returned as a ``Structure`` with a row-vector ``lattice`` [3,3]
(row v = lattice vector v, the convention of MatPL's loader and ``NeighConst.f90:66``),
fractional ``frac`` [N,3], Cartesian ``cart`` [N,3] and 0-based ``types`` [N] sorted so
that atoms of one element are contiguous (MatPL's images list atoms grouped by element).
"""
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np


@dataclass
class Structure:
    lattice: np.ndarray      # [3,3] f64, rows are lattice vectors (Angstrom)
    frac: np.ndarray         # [N,3] f64 fractional coordinates in [0,1)
    types: np.ndarray        # [N] int32, 0-based index into ``elements``
    elements: List[int]      # atomic numbers, in type order

    @property
    def natoms(self) -> int:
        return int(self.frac.shape[0])

    @property
    def cart(self) -> np.ndarray:
        return self.frac @ self.lattice


def fcc(a: float, reps: Sequence[int], sigma: float, seed: int, element: int = 29) -> Structure:
    """FCC crystal of ``reps`` conventional cells, displaced by N(0, sigma^2) per component."""
    rng = np.random.default_rng(seed)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], dtype=np.float64)
    nx, ny, nz = reps
    cells = np.array([[i, j, k] for i in range(nx) for j in range(ny) for k in range(nz)],
                     dtype=np.float64)
    frac = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) / np.array([nx, ny, nz])
    lattice = np.diag([a * nx, a * ny, a * nz]).astype(np.float64)
    cart = frac @ lattice + rng.normal(0.0, sigma, size=frac.shape)
    frac = np.mod(cart @ np.linalg.inv(lattice), 1.0)
    return Structure(lattice, frac, np.zeros(len(frac), dtype=np.int32), [element])


def random_packed(natoms: int, density: float, elements: Sequence[int],
                  fractions: Sequence[float], seed: int, min_dist: float = 2.0,
                  strain: float = 0.0) -> Structure:
    """Random insertion of ``natoms`` atoms in a cube of the given number density
    (atoms / A^3) with all periodic pair distances >= ``min_dist``, then an optional symmetric
    strain eps with entries N(0, strain) applied to the cell (cell = cube (I + eps)).

    Candidates are drawn in seeded batches and checked on a grid of cells of edge
    <= min_dist/sqrt(3) (at most one atom per cell): a candidate is rejected if an accepted
    atom, or an earlier candidate of its own batch, lies closer than ``min_dist``.
    Element counts follow ``fractions`` (rounded, remainder to the last element)."""
    rng = np.random.default_rng(seed)
    L = (natoms / density) ** (1.0 / 3.0)
    nb = max(1, int(np.ceil(L / (min_dist / np.sqrt(3.0)))))
    w = L / nb
    reach = int(np.ceil(min_dist / w))
    rr = np.arange(-reach, reach + 1)
    offs = np.stack(np.meshgrid(rr, rr, rr, indexing="ij"), -1).reshape(-1, 3)
    grid = -np.ones((nb, nb, nb), dtype=np.int64)
    pts = np.empty((natoms, 3), dtype=np.float64)
    md2 = min_dist * min_dist
    n = 0
    rounds = 0

    def conflicts(cand, cells, g, src):
        nc = (cells[:, None, :] + offs[None, :, :]) % nb
        occ = g[nc[..., 0], nc[..., 1], nc[..., 2]]                 # [B, K]
        ok = occ >= 0
        d = src[np.where(ok, occ, 0)] - cand[:, None, :]
        d -= L * np.round(d / L)
        close = ok & (np.einsum("bkj,bkj->bk", d, d) < md2)
        return close, occ

    while n < natoms:
        rounds += 1
        if rounds > 10000:
            raise RuntimeError("random_packed: insertion stalled; lower density or min_dist")
        bsz = int(min(8192, max(64, 2 * (natoms - n))))
        cand = rng.random((bsz, 3)) * L
        cells = np.minimum((cand / w).astype(np.int64), nb - 1)
        close, _ = conflicts(cand, cells, grid, pts)
        keep = ~close.any(1)
        cand, cells = cand[keep], cells[keep]
        if len(cand) == 0:
            continue
        # intra-batch: drop a candidate that conflicts with an earlier one of the batch
        tg = -np.ones((nb, nb, nb), dtype=np.int64)
        order = np.arange(len(cand))
        tg[cells[::-1, 0], cells[::-1, 1], cells[::-1, 2]] = order[::-1]   # earliest wins a cell
        same_cell_loser = tg[cells[:, 0], cells[:, 1], cells[:, 2]] != order
        close_b, occ_b = conflicts(cand, cells, tg, cand)
        earlier = close_b & (occ_b < order[:, None])
        keep = ~(earlier.any(1) | same_cell_loser)
        cand, cells = cand[keep], cells[keep]
        take = min(len(cand), natoms - n)
        cand, cells = cand[:take], cells[:take]
        pts[n:n + take] = cand
        grid[cells[:, 0], cells[:, 1], cells[:, 2]] = np.arange(n, n + take)
        n += take
    counts = [int(round(f * natoms)) for f in fractions[:-1]]
    counts.append(natoms - sum(counts))
    types = np.concatenate([np.full(c, t, dtype=np.int32) for t, c in enumerate(counts)])
    lattice = np.eye(3) * L
    if strain > 0.0:
        e = rng.normal(0.0, strain, size=(3, 3))
        e = 0.5 * (e + e.T)
        lattice = lattice @ (np.eye(3) + e)
    frac = np.mod(pts / L, 1.0)
    return Structure(lattice, frac, types, list(elements))


def maxwell_boltzmann(masses_amu: np.ndarray, temperature_k: float, seed: int) -> np.ndarray:
    """Velocities (A/fs) drawn from the Maxwell-Boltzmann distribution, net momentum removed."""
    rng = np.random.default_rng(seed)
    kb_ev = 8.617333262e-5
    amu_ev_fs2_a2 = 103.642696562  # 1 amu A^2 / fs^2 = 103.64 eV
    sig = np.sqrt(kb_ev * temperature_k / (masses_amu * amu_ev_fs2_a2))
    v = rng.normal(size=(len(masses_amu), 3)) * sig[:, None]
    p = (v * masses_amu[:, None]).sum(0) / masses_amu.sum()
    return v - p
