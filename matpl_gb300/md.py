"""Batched molecular dynamics of many independent replicas with one DP model.

All replicas live in one ragged atom array (replica r owns a contiguous range of atoms), so
every part of a step is one launch over every replica, whatever their sizes:

1. ``matpl_md_drift``: x += v dt + a dt^2 / 2, and the rebuild flag when an atom has moved
   more than skin / 2 since the last list build (the displacement rule of the LAMMPS loop
   around the pair style, pair_matpl.cpp:1096-1110);
2. ``matpl_md_skin_build``: the Verlet list at Rc + skin (default skin 1.0 A) of every replica,
   run only when the flag is set - the decision is taken on the device, so a captured step
   needs no host round trip;
3. ``matpl_md_skin_filter``: the pairs inside Rc at the current positions as the occupied-slot
   list of one image of all atoms (global neighbor indices);
4. ``matpl_dp_eval_occupied`` (``DP.evaluate(..., num_neigh=...)``): fused E/F/V of all
   replicas in one evaluation;
5. ``matpl_md_kick``: the closing half kick and the per-replica kinetic / potential energies
   (FP64, fixed summation order).

The step is captured once as a CUDA graph (``steps_per_graph`` steps per graph) and replayed.
A pair between Rc and Rc + skin is left out of the filtered list, so the evaluation counts it
among its type block's empty slots, exactly as an exact search at the same positions would: the
forces do not depend on when the list was built.  The energy record gives the drift of the
total energy per replica.

Units: Angstrom, fs, amu, eV (1 amu A^2 / fs^2 = 103.6427 eV).
"""
import math
from typing import Dict, Optional, Sequence

import numpy as np
import torch

from . import _lib, dp as _dp
from ._lib import check, ptr
from .params import DPConfig
from .structures import Structure, maxwell_boltzmann

AMU_A2_FS2_EV = 103.642696562
BUILD_BLOCK = 128        # atoms per block of matpl_md_skin_build


class ReplicaMD:
    def __init__(self, cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
                 replicas: Sequence[Structure], masses_amu: Sequence[float], dt_fs: float = 1.0,
                 temperature_k: float = 300.0, precision: str = "mixed", seed: int = 0,
                 device="cuda", skin: float = 1.0, skin_capacity: Optional[int] = None,
                 steps_per_graph: int = 1):
        self.cfg = cfg
        self.dev = torch.device(device)
        if self.dev.index is None:
            self.dev = torch.device("cuda", torch.cuda.current_device())
        self.dt = float(dt_fs)
        self.skin = float(skin)
        self.steps_per_graph = max(1, int(steps_per_graph))
        self.model = _dp.DP(cfg, params, davg, dstd, precision=precision, device=self.dev,
                            check_errors=False)
        self.present = self.model.present_types(cfg.atom_type)
        T, m = cfg.ntypes, cfg.maxNeighborNum
        self.rc = float(cfg.Rmax)
        # skin-list capacity per type block: the Rc block scaled by the shell volume, + 15 %
        self.cap = int(skin_capacity or 4 * math.ceil(
            m * ((self.rc + self.skin) / self.rc) ** 3 * 1.15 / 4))
        masses = np.asarray(masses_amu, dtype=np.float64)
        counts = np.array([st.natoms for st in replicas], dtype=np.int64)
        start = np.zeros(len(replicas) + 1, dtype=np.int64)
        start[1:] = np.cumsum(counts)
        ntot = int(start[-1])
        types = np.concatenate([np.asarray(st.types, dtype=np.int32) for st in replicas])
        x = np.concatenate([np.asarray(st.cart, dtype=np.float64) for st in replicas])
        m_at = masses[types]
        v = np.concatenate([maxwell_boltzmann(masses[np.asarray(st.types)], temperature_k,
                                              seed + r) for r, st in enumerate(replicas)])
        lat = np.stack([np.asarray(st.lattice, dtype=np.float64) for st in replicas])
        work = np.array([(r, i0) for r in range(len(replicas))
                         for i0 in range(0, int(counts[r]), BUILD_BLOCK)], dtype=np.int32)
        d, f64, i32 = self.dev, torch.float64, torch.int32
        t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=d)  # noqa: E731
        self.counts = counts
        self._start = start
        self.nreplicas = len(replicas)
        self.natoms_total = ntot
        self.rep_start = t(start, i32)
        self.atom_rep = t(np.repeat(np.arange(len(replicas)), counts), i32)
        self.work = t(work.reshape(-1), i32)
        self.nwork = int(work.shape[0])
        self.types = t(types, i32)
        self.lat = t(lat, f64)
        self.inv_lat = t(np.linalg.inv(lat), f64)
        self.x = t(x, f64)
        self.v = t(v, f64)
        self.a = torch.zeros(ntot, 3, dtype=f64, device=d)
        self.mass = t(m_at, f64)
        self.inv_mass = t(1.0 / (m_at * AMU_A2_FS2_EV), f64)
        self.x_ref = torch.zeros(ntot, 3, dtype=f64, device=d)
        self.nbr = torch.zeros(ntot, T * self.cap, dtype=i32, device=d)
        self.img = torch.zeros(ntot, T * self.cap, dtype=i32, device=d)
        self.cnt = torch.zeros(ntot, T, dtype=i32, device=d)
        self.gate = torch.ones(1, dtype=i32, device=d)       # the first step builds the list
        self.nbuild = torch.zeros(1, dtype=i32, device=d)
        self.err = torch.zeros(1, dtype=i32, device=d)
        S = T * m
        self.ln = torch.zeros(1, ntot, S, dtype=i32, device=d)
        self.idr = torch.zeros(1, ntot, S, 4, dtype=self.model.dtype, device=d)
        self.nn = torch.zeros(1, ntot, T, dtype=i32, device=d)
        self.out = {"Ei_atom": torch.empty(1, ntot, dtype=self.model.dtype, device=d),
                    "Etot": torch.empty(1, dtype=f64, device=d),
                    "Force": torch.empty(1, ntot, 3, dtype=self.model.dtype, device=d),
                    "Virial": torch.empty(1, 9, dtype=f64, device=d)}
        self.ke = torch.zeros(self.nreplicas, dtype=f64, device=d)
        self.pe = torch.zeros(self.nreplicas, dtype=f64, device=d)
        self._code = _lib.MATPL_F64 if self.model.dtype == torch.float64 else _lib.MATPL_F32
        self.graph = None
        with torch.cuda.device(self.dev):
            self._forces()
            self._kick(0)

    # -------------------------------------------------------------------------- one step
    def _stream(self):
        return torch.cuda.current_stream(self.dev).cuda_stream

    def _forces(self):
        lib = _lib.load()
        cfg = self.cfg
        st = self._stream()
        check(lib.matpl_md_skin_build(
            self.nreplicas, self.natoms_total, cfg.ntypes, self.cap, self.rc + self.skin,
            ptr(self.rep_start), ptr(self.work), self.nwork, ptr(self.lat), ptr(self.inv_lat),
            ptr(self.types), ptr(self.x), ptr(self.nbr), ptr(self.img), ptr(self.cnt),
            ptr(self.x_ref), ptr(self.gate), ptr(self.nbuild), ptr(self.err), st),
            "matpl_md_skin_build")
        check(lib.matpl_md_skin_filter(
            self._code, self.natoms_total, cfg.ntypes, self.cap, cfg.maxNeighborNum, self.rc,
            ptr(self.atom_rep), ptr(self.lat), ptr(self.nbr), ptr(self.img), ptr(self.cnt),
            ptr(self.x), ptr(self.ln), ptr(self.idr), ptr(self.nn), ptr(self.err), st),
            "matpl_md_skin_filter")
        self.model.evaluate(self.ln, self.types, self.present, self.idr, 0, out=self.out,
                            num_neigh=self.nn)

    def _kick(self, mode: int):
        check(_lib.load().matpl_md_kick(
            self._code, mode, self.nreplicas, self.dt, AMU_A2_FS2_EV, ptr(self.rep_start),
            ptr(self.inv_mass), ptr(self.mass), ptr(self.out["Force"]), ptr(self.out["Ei_atom"]),
            ptr(self.v), ptr(self.a), ptr(self.ke), ptr(self.pe), self._stream()), "matpl_md_kick")

    def _step(self):
        check(_lib.load().matpl_md_drift(self.natoms_total, self.dt, self.skin, ptr(self.x),
                                         ptr(self.v), ptr(self.a), ptr(self.x_ref),
                                         ptr(self.gate), self._stream()), "matpl_md_drift")
        self._forces()
        self._kick(1)

    # -------------------------------------------------------------------------- driver
    _STATE = ("x", "v", "a", "ke", "pe", "x_ref", "nbr", "img", "cnt", "gate", "nbuild")

    def capture(self, warmup: int = 2):
        """Capture ``steps_per_graph`` steps; the warm-up steps that precede the capture (they
        settle the allocator and the kernels' attributes) leave the trajectory unchanged."""
        keep = {k: getattr(self, k).clone() for k in self._STATE}
        keep_out = {k: t.clone() for k, t in self.out.items()}
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            for _ in range(warmup):
                self._step()
        torch.cuda.current_stream(self.dev).wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=side):
            for _ in range(self.steps_per_graph):
                self._step()
        for k, t in keep.items():
            getattr(self, k).copy_(t)
        for k, t in keep_out.items():
            self.out[k].copy_(t)

    def step(self, n: int = 1):
        """n steps of every replica: n // steps_per_graph graph launches, the rest eagerly."""
        if self.graph is None:
            self.capture()
        for _ in range(n // self.steps_per_graph):
            self.graph.replay()
        with torch.cuda.device(self.dev):
            for _ in range(n % self.steps_per_graph):
                self._step()

    def energies(self) -> np.ndarray:
        """[replicas, 2] (potential, kinetic) in eV, in the order the replicas were given."""
        return torch.stack([self.pe, self.ke], 1).cpu().numpy()

    def rebuilds(self) -> int:
        """Skin-list builds so far (the first one included)."""
        return int(self.nbuild.item())

    def check_errors(self):
        code = int(self.err.item()) or int(self.model.err.item())
        if code:
            raise _lib.MatplError(f"MD kernels reported error code {code} (1 = neighbor "
                                  "overflow, 4 = cell or image range)")

    def natoms(self) -> np.ndarray:
        return self.counts.copy()

    def replica_slice(self, r: int) -> slice:
        """Rows of replica r in the ragged atom arrays (x, v, a, out["Force"][0], ...)."""
        return slice(int(self._start[r]), int(self._start[r + 1]))
