"""NEP model description on the host: hyper-parameters, parameters, periodic box expansion.

Mirrors the parts of MatPL that the NEP evaluation path reads:

* ``NepConfig``: ``NepParam`` (src/user/nep_param.py:51-83) - cutoff [radial, angular], n_max,
  basis_size, l_max [3-body, 4-body, 5-body], neuron [hidden, 1], train_2b - plus the element
  list; ``feature_nums`` follows ``NEP.set_init_nep_param`` (src/model/nep_net.py:111-143).
* ``init_params``: seeded parameters of the shapes ``NEP`` holds - ``c_param_2``
  [T, T, n_max_r + 1, basis_r + 1], ``c_param_3`` [T, T, n_max_a + 1, basis_a + 1]
  (nep_net.py:160-176), one single-hidden-layer ``FittingNet`` per element
  (src/model/nep_fitting.py:40-95) and ``q_scaler`` [F].
* ``calc_q_scaler``: ``NEP.update_scaler_values`` (nep_net.py:1020-1058), q_scaler = 1/(max-min)
  with shared extrema over each (l, body-order) block.
* ``expand_box``: ``UniDataset.expand_box`` (src/pre_data/nep_data_loader.py:220-253): the number
  of replicas per lattice direction, the replicated cell h (columns = vectors) and h^-1.
* ``pack_params``: the flat device layout of ``matpl_nep_eval``.
"""
from dataclasses import dataclass, field
from typing import Dict, List, Sequence

import math

import numpy as np
import torch


@dataclass
class NepConfig:
    atom_type: List[int]
    cutoff: Sequence[float] = (6.0, 4.0)
    n_max: Sequence[int] = (4, 4)
    basis_size: Sequence[int] = (8, 8)
    l_max: Sequence[int] = (4, 2, 1)
    neuron: int = 30
    train_2b: bool = True

    @property
    def ntypes(self) -> int:
        return len(self.atom_type)

    @property
    def nr(self) -> int:          # radial descriptor components n = 0..n_max_r
        return self.n_max[0] + 1

    @property
    def na(self) -> int:          # angular radial functions n = 0..n_max_a
        return self.n_max[1] + 1

    @property
    def kr(self) -> int:          # Chebyshev basis functions k = 0..basis_r
        return self.basis_size[0] + 1

    @property
    def ka(self) -> int:
        return self.basis_size[1] + 1

    @property
    def two_feat_num(self) -> int:
        return self.nr if self.train_2b else 0

    @property
    def multi_feat_num(self) -> int:
        l3, l4, l5 = self.l_max
        if l3 <= 0:
            return 0
        return self.na * l3 + (self.na if l4 > 0 else 0) + (self.na if l5 > 0 else 0)

    @property
    def feature_nums(self) -> int:
        return self.two_feat_num + self.multi_feat_num


def init_params(cfg: NepConfig, seed: int, energy_shift: float = 0.0,
                dtype=torch.float64) -> Dict[str, torch.Tensor]:
    """Seeded parameters with the reference's shapes and initial distributions: c = U(-0.5, 0.5)
    + 0.1 N(0, 1) (nep_net.py:166-170); hidden weight N(0, 1/sqrt(F + H)), bias N(0, 1); output
    weight N(0, 1/sqrt(H + 1)), bias N(energy_shift, 1) (nep_fitting.py:62-91).  q_scaler is set
    to 1; ``calc_q_scaler`` replaces it from descriptor statistics."""
    g = torch.Generator().manual_seed(seed)
    T, F, H = cfg.ntypes, cfg.feature_nums, cfg.neuron

    def cparam(n, k):
        m = torch.rand(T, T, n, k, generator=g, dtype=torch.float64) - 0.5
        return m + 0.1 * torch.randn(T, T, n, k, generator=g, dtype=torch.float64)

    p = {"c_param_2": cparam(cfg.nr, cfg.kr)}
    if cfg.l_max[0] > 0:
        p["c_param_3"] = cparam(cfg.na, cfg.ka)
    for t in range(T):
        pre = f"fitting_net.{t}.layers."
        p[pre + "0.weight"] = torch.randn(F, H, generator=g, dtype=torch.float64) / math.sqrt(F + H)
        p[pre + "0.bias"] = torch.randn(1, H, generator=g, dtype=torch.float64)
        p[pre + "1.weight"] = torch.randn(H, 1, generator=g, dtype=torch.float64) / math.sqrt(H + 1)
        p[pre + "1.bias"] = energy_shift + torch.randn(1, 1, generator=g, dtype=torch.float64)
    p["q_scaler"] = torch.ones(F, dtype=torch.float64)
    return {k: v.to(dtype) for k, v in p.items()}


def scaler_blocks(cfg: NepConfig):
    """Column ranges that share one extremum in ``update_scaler_values`` (nep_net.py:1027-1043):
    the radial block, one block per l of the 3-body part, the 4-body and the 5-body blocks."""
    blocks = [(0, cfg.two_feat_num)]
    off = cfg.two_feat_num
    l3, l4, l5 = cfg.l_max
    if l3 > 0:
        for _ in range(l3):
            blocks.append((off, off + cfg.na))
            off += cfg.na
        if l4 > 0:
            blocks.append((off, off + cfg.na))
            off += cfg.na
        if l5 > 0:
            blocks.append((off, off + cfg.na))
    return [b for b in blocks if b[1] > b[0]]


def calc_q_scaler(cfg: NepConfig, feats: torch.Tensor) -> torch.Tensor:
    """q_scaler = 1 / (q_max - q_min), extrema taken per block over all atoms."""
    f = feats.reshape(-1, feats.shape[-1])
    qmax = f.max(0).values.clone()
    qmin = f.min(0).values.clone()
    for a, b in scaler_blocks(cfg):
        qmax[a:b] = qmax[a:b].max()
        qmin[a:b] = qmin[a:b].min()
    return 1.0 / (qmax - qmin)


def _det3(m: np.ndarray) -> float:
    return float(np.linalg.det(m.reshape(3, 3)))


def expand_box(lattice: np.ndarray, cutoff_radial: float):
    """(box [18], box_orig [9], num_cell [3], volume) for one frame.

    ``lattice`` has the lattice vectors as rows.  box_orig = lattice^T flattened, box[0:9] the
    replicated cell h with columns num_cell[k] * vector k, box[9:18] = adj(h) / det(h)."""
    lat = np.asarray(lattice, dtype=np.float64).reshape(3, 3)
    lt = lat.T.flatten()
    a, b, c = lt[0::3], lt[1::3], lt[2::3]

    def area(u, v):
        s1 = u[1] * v[2] - u[2] * v[1]
        s2 = u[2] * v[0] - u[0] * v[2]
        s3 = u[0] * v[1] - u[1] * v[0]
        return math.sqrt(s1 * s1 + s2 * s2 + s3 * s3)

    det = _det3(lt)
    volume = abs(det)
    num_cell = np.array([int(math.ceil(2.0 * cutoff_radial / (volume / area(b, c)))),
                         int(math.ceil(2.0 * cutoff_radial / (volume / area(c, a)))),
                         int(math.ceil(2.0 * cutoff_radial / (volume / area(a, b))))],
                        dtype=np.int64)
    box = np.zeros(18, dtype=np.float64)
    box[0:9:3] = lt[0::3] * num_cell[0]
    box[1:9:3] = lt[1::3] * num_cell[1]
    box[2:9:3] = lt[2::3] * num_cell[2]
    box[9] = box[4] * box[8] - box[5] * box[7]
    box[10] = box[2] * box[7] - box[1] * box[8]
    box[11] = box[1] * box[5] - box[2] * box[4]
    box[12] = box[5] * box[6] - box[3] * box[8]
    box[13] = box[0] * box[8] - box[2] * box[6]
    box[14] = box[2] * box[3] - box[0] * box[5]
    box[15] = box[3] * box[7] - box[4] * box[6]
    box[16] = box[1] * box[6] - box[0] * box[7]
    box[17] = box[0] * box[4] - box[1] * box[3]
    det *= float(num_cell[0] * num_cell[1] * num_cell[2])
    box[9:18] /= det
    return box, lt.copy(), num_cell, volume


@dataclass
class NepFrames:
    """A batch of frames in the reference's concatenated-atoms layout (nep_data_loader.py:200-215
    with ``variable_length_collate_fn``): cartesian positions [sum N, 3], per-atom element index,
    per-frame atom counts, box [B, 18], box_orig [B, 9], num_cell [B, 3]."""
    position: np.ndarray
    type_map: np.ndarray
    num_atom: np.ndarray
    box: np.ndarray
    box_orig: np.ndarray
    num_cell: np.ndarray
    volume: np.ndarray = field(default=None)

    @property
    def natoms(self) -> int:
        return int(self.position.shape[0])

    @property
    def nframes(self) -> int:
        return int(self.num_atom.shape[0])


def frames_from_structures(structs, cutoff_radial: float) -> NepFrames:
    """Concatenate ``matpl_gb300.structures.Structure`` objects (row-vector lattices, fractional
    coordinates, element indices) into the reference's NEP batch layout."""
    pos, tm, na, bx, bo, nc, vol = [], [], [], [], [], [], []
    for st in structs:
        box, lt, ncell, v = expand_box(st.lattice, cutoff_radial)
        pos.append(st.frac @ st.lattice)
        tm.append(np.asarray(st.types, dtype=np.int64))
        na.append(st.natoms)
        bx.append(box); bo.append(lt); nc.append(ncell); vol.append(v)
    return NepFrames(np.concatenate(pos), np.concatenate(tm), np.array(na, dtype=np.int64),
                     np.stack(bx), np.stack(bo), np.stack(nc), np.array(vol))


# ----------------------------------------------------------------------------------------------
# flat parameter layout of matpl_nep_eval (one contiguous buffer of the compute dtype):
#   c2 [T, T, nr, kr] | c3 [T, T, na, ka] | q_scaler [F] |
#   per type t: W0 [F, H] | b0 [H] | W1 [H] | b1 [1]
# ----------------------------------------------------------------------------------------------
def param_count(cfg: NepConfig) -> int:
    T, F, H = cfg.ntypes, cfg.feature_nums, cfg.neuron
    n = T * T * cfg.nr * cfg.kr + (T * T * cfg.na * cfg.ka if cfg.l_max[0] > 0 else 0) + F
    return n + T * (F * H + 2 * H + 1)


def pack_params(cfg: NepConfig, p: Dict[str, torch.Tensor]) -> torch.Tensor:
    parts = [p["c_param_2"].reshape(-1)]
    if cfg.l_max[0] > 0:
        parts.append(p["c_param_3"].reshape(-1))
    parts.append(p["q_scaler"].reshape(-1))
    for t in range(cfg.ntypes):
        pre = f"fitting_net.{t}.layers."
        parts += [p[pre + "0.weight"].reshape(-1), p[pre + "0.bias"].reshape(-1),
                  p[pre + "1.weight"].reshape(-1), p[pre + "1.bias"].reshape(-1)]
    flat = torch.cat([x.detach().to(torch.float64).cpu() for x in parts])
    assert flat.numel() == param_count(cfg)
    return flat
