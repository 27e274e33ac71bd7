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
    """Random sequential insertion of ``natoms`` atoms in a cube of the given number density
    (atoms / A^3) with all pair distances >= ``min_dist`` (periodic), then an optional
    symmetric strain eps with entries N(0, strain) applied to the cell (cell = cube (I + eps)).
    Element counts follow ``fractions`` (rounded, remainder to the last element)."""
    rng = np.random.default_rng(seed)
    L = (natoms / density) ** (1.0 / 3.0)
    nb = max(1, int(L // min_dist))
    w = L / nb
    grid = {}
    pts = np.empty((natoms, 3), dtype=np.float64)
    n = 0
    md2 = min_dist * min_dist
    attempts = 0
    while n < natoms:
        cand = rng.random((256, 3)) * L
        for p in cand:
            attempts += 1
            if attempts > 200 * natoms + 10000:
                raise RuntimeError("random_packed: insertion stalled; lower density or min_dist")
            c = np.floor(p / w).astype(int) % nb
            ok = True
            for dx in (-1, 0, 1):
                if not ok:
                    break
                for dy in (-1, 0, 1):
                    if not ok:
                        break
                    for dz in (-1, 0, 1):
                        key = ((c[0] + dx) % nb, (c[1] + dy) % nb, (c[2] + dz) % nb)
                        lst = grid.get(key)
                        if not lst:
                            continue
                        d = pts[lst] - p
                        d -= L * np.round(d / L)
                        if np.any(np.einsum("ij,ij->i", d, d) < md2):
                            ok = False
                            break
            if ok:
                pts[n] = p
                grid.setdefault((c[0], c[1], c[2]), []).append(n)
                n += 1
                if n == natoms:
                    break
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
