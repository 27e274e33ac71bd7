"""Batched molecular dynamics of many independent replicas with one DP model.

Replicas of uneven atom counts are grouped by (atom count, element sequence) into [B, N]
batches; every group keeps its positions, velocities, neighbor list, environment data and
outputs in persistent device buffers.  One MD step of *all* replicas - velocity-Verlet drift,
neighbor search (``matpl_neighbor_build``), fused E/F/V (``matpl_dp_eval``) and the velocity
update - is captured once as a CUDA graph and replayed, so a step costs one graph launch
whatever the number of replicas.  The neighbor lists are rebuilt every step from the exact
search (a Verlet skin would give the same forces: slots between Rc and Rc + skin carry s = 0 and
act exactly like empty slots, but rebuilding costs less than tracking periodic-image shifts
for the small cells).  Energies and the virial are summed in FP64; the energy record gives the
drift of the total energy per replica.

Units: Angstrom, fs, amu, eV (1 amu A^2 / fs^2 = 103.6427 eV).
"""
import ctypes
from typing import Dict, List, Sequence

import numpy as np
import torch

from . import _lib, dp as _dp, ops
from ._lib import check, ptr
from .params import DPConfig
from .structures import Structure, maxwell_boltzmann

AMU_A2_FS2_EV = 103.642696562


class ReplicaMD:
    def __init__(self, cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
                 replicas: Sequence[Structure], masses_amu: Sequence[float], dt_fs: float = 1.0,
                 temperature_k: float = 300.0, precision: str = "mixed", seed: int = 0,
                 device="cuda"):
        self.cfg = cfg
        self.dev = torch.device(device)
        self.dt = float(dt_fs)
        self.model = _dp.DP(cfg, params, davg, dstd, precision=precision, device=self.dev,
                            check_errors=False)
        self.present = self.model.present_types(cfg.atom_type)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.rct = (ctypes.c_double * cfg.ntypes)(*([float(cfg.Rmax)] * cfg.ntypes))
        masses = np.asarray(masses_amu, dtype=np.float64)
        keyed: Dict[tuple, List[int]] = {}
        for r, st in enumerate(replicas):
            keyed.setdefault((st.natoms, tuple(st.types.tolist())), []).append(r)
        self.groups = []
        S = cfg.ntypes * cfg.maxNeighborNum
        lib = _lib.load()
        nb_ws = dp_ws = 0
        for (N, types), idx in sorted(keyed.items()):
            B = len(idx)
            lat = np.stack([replicas[r].lattice for r in idx])
            x = np.stack([replicas[r].cart for r in idx])
            m = masses[np.asarray(types)]
            v = np.stack([maxwell_boltzmann(m, temperature_k, seed + r) for r in idx])
            g = {"idx": idx, "B": B, "N": N,
                 "types": torch.tensor(types, dtype=torch.int32, device=self.dev),
                 "lat": torch.tensor(lat, device=self.dev),
                 "inv_lat": torch.tensor(np.linalg.inv(lat), device=self.dev),
                 "x": torch.tensor(x, device=self.dev), "v": torch.tensor(v, device=self.dev),
                 "m": torch.tensor(m, device=self.dev).reshape(1, N, 1),
                 "frac": torch.empty(B, N, 3, dtype=torch.float64, device=self.dev),
                 "ln": torch.empty(B, N, S, dtype=torch.int32, device=self.dev),
                 "idr": torch.empty(B, N, S, 4, dtype=self.model.dtype, device=self.dev),
                 "out": {"Ei_atom": torch.empty(B, N, dtype=self.model.dtype, device=self.dev),
                         "Etot": torch.empty(B, dtype=torch.float64, device=self.dev),
                         "Force": torch.empty(B, N, 3, dtype=self.model.dtype, device=self.dev),
                         "Virial": torch.empty(B, 9, dtype=torch.float64, device=self.dev)},
                 "a": torch.zeros(B, N, 3, dtype=torch.float64, device=self.dev),
                 "ke": torch.zeros(B, dtype=torch.float64, device=self.dev)}
            nb_ws = max(nb_ws, lib.matpl_neighbor_workspace_bytes(B, N))
            dp_ws = max(dp_ws, lib.matpl_dp_workspace_bytes(self.model.code, B, N))
            self.groups.append(g)
        # the neighbor workspace is sized once for the largest group and owned here; the
        # evaluation's workspace is sized on the capture stream before the capture
        self.nb_ws = ops.workspace(self.dev, nb_ws, "neighbor")
        self._dp_ws_bytes = dp_ws
        self.natoms_total = sum(g["B"] * g["N"] for g in self.groups)
        self.nreplicas = len(replicas)
        self.graph = None
        for g in self.groups:
            self._forces(g)
            g["a"].copy_(self._accel(g))
            self._kinetic(g)

    # -------------------------------------------------------------------------- one group
    def _forces(self, g):
        cfg = self.cfg
        B, N = g["B"], g["N"]
        torch.matmul(g["x"], g["inv_lat"], out=g["frac"])
        with torch.cuda.device(self.dev):
            check(_lib.load().matpl_neighbor_build(
                B, N, cfg.ntypes, cfg.maxNeighborNum, float(cfg.Rmax), self.rct, ptr(g["types"]),
                ptr(g["lat"]), ptr(g["frac"]), self.model.code if self.model.code in (0, 1) else 0,
                ptr(g["ln"]), ptr(g["idr"]), 0, ptr(self.err), ptr(self.nb_ws),
                self.nb_ws.numel(), torch.cuda.current_stream(self.dev).cuda_stream),
                "matpl_neighbor_build")
        self.model.evaluate(g["ln"], g["types"], self.present, g["idr"], 0, out=g["out"])

    def _accel(self, g):
        return g["out"]["Force"].to(torch.float64) / (g["m"] * AMU_A2_FS2_EV)

    def _kinetic(self, g):
        ke = 0.5 * AMU_A2_FS2_EV * (g["m"] * g["v"] * g["v"]).sum((1, 2))
        g["ke"].copy_(ke)

    def _step(self):
        dt = self.dt
        for g in self.groups:
            g["x"].add_(g["v"] * dt + 0.5 * dt * dt * g["a"])
            self._forces(g)
            a_new = self._accel(g)
            g["v"].add_(0.5 * dt * (g["a"] + a_new))
            g["a"].copy_(a_new)
            self._kinetic(g)

    # -------------------------------------------------------------------------- driver
    def capture(self, warmup: int = 2):
        """Capture one step of every group; the warm-up steps that precede the capture (they
        settle the allocator and the kernels' attributes) leave the trajectory unchanged."""
        keep = [{k: g[k].clone() for k in ("x", "v", "a", "ke")} for g in self.groups]
        keep_out = [{k: t.clone() for k, t in g["out"].items()} for g in self.groups]
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            ops.workspace(self.dev, self._dp_ws_bytes, "dp")   # nothing grows in the capture
            for _ in range(warmup):
                self._step()
        torch.cuda.current_stream(self.dev).wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=side):
            self._step()
        for g, kp, ko in zip(self.groups, keep, keep_out):
            for k, t in kp.items():
                g[k].copy_(t)
            for k, t in ko.items():
                g["out"][k].copy_(t)

    def step(self, n: int = 1):
        if self.graph is None:
            self.capture()
        for _ in range(n):
            self.graph.replay()

    def energies(self) -> np.ndarray:
        """[replicas, 2] (potential, kinetic) in eV, in the order the replicas were given."""
        out = np.zeros((self.nreplicas, 2))
        for g in self.groups:
            pe = g["out"]["Etot"].cpu().numpy()
            ke = g["ke"].cpu().numpy()
            for b, r in enumerate(g["idx"]):
                out[r] = (pe[b], ke[b])
        return out

    def check_errors(self):
        code = int(self.err.item()) or int(self.model.err.item())
        if code:
            raise _lib.MatplError(f"MD kernels reported error code {code} (1 = neighbor overflow)")

    def natoms(self) -> np.ndarray:
        n = np.zeros(self.nreplicas, dtype=np.int64)
        for g in self.groups:
            for r in g["idx"]:
                n[r] = g["N"]
        return n
