"""DP se_e2_a model description, parameter initialisation and the davg/dstd statistics.

The parameter dictionary uses the reference's own ``state_dict`` key names
(``src/model/dp_dp.py:69-85``, ``src/model/dp_embedding.py:30-138``):

    embedding_net.{ti*ntypes+tj}.layers.{l}.{weight,bias[,resnet_dt]}   l = 0..len(emb)-1
    fitting_net.{ti}.layers.{l}.{weight,bias[,resnet_dt]}                l = 0..len(fit)-1

so checkpoints and TorchScript exports of the reference load directly
(``load_reference_state_dict``).
"""
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import torch


@dataclass
class DPConfig:
    """Hyper-parameters read by ``DP.__init__`` (``dp_dp.py:44-85``)."""
    atom_type: List[int]                      # model element list (atomic numbers)
    Rmax: float = 6.0                         # config["Rc_M"]
    Rmin: float = 0.5                         # config["atomType"][0]["Rm"]
    maxNeighborNum: int = 100                 # m: slots per neighbor type
    M2: int = 16
    emb_sizes: List[int] = field(default_factory=lambda: [25, 25, 25])
    fit_sizes: List[int] = field(default_factory=lambda: [50, 50, 50, 1])
    emb_resnet_dt: bool = False               # reference default (nn_feature_type.py:10-29)
    fit_resnet_dt: bool = True

    @property
    def ntypes(self) -> int:
        return len(self.atom_type)

    @property
    def nslots(self) -> int:
        return self.ntypes * self.maxNeighborNum


def init_params(cfg: DPConfig, seed: int, energy_shift: Optional[List[float]] = None,
                dtype=torch.float64) -> Dict[str, torch.Tensor]:
    """Random weights W ~ N(0, 1/fan_in), biases ~ N(0, 0.1^2), resnet_dt ~ N(0.1, 0.001^2)
    (fitting) or N(1, 0.001^2) (embedding), last fitting bias = energy_shift[t]."""
    rng = np.random.default_rng(seed)
    p: Dict[str, torch.Tensor] = {}
    nt = cfg.ntypes
    shift = energy_shift if energy_shift is not None else [0.0] * nt

    def t(a):
        return torch.tensor(np.asarray(a, dtype=np.float64), dtype=dtype)

    widths = [1] + list(cfg.emb_sizes)
    for k in range(nt * nt):
        for l in range(len(cfg.emb_sizes)):
            fi, fo = widths[l], widths[l + 1]
            pre = f"embedding_net.{k}.layers.{l}."
            p[pre + "weight"] = t(rng.normal(0, 1 / np.sqrt(fi), (fi, fo)))
            p[pre + "bias"] = t(rng.normal(0, 0.1, (1, fo)))
            if cfg.emb_resnet_dt:
                p[pre + "resnet_dt"] = t(rng.normal(1.0, 0.001, (1, fo)))
    fw = [cfg.M2 * cfg.emb_sizes[-1]] + list(cfg.fit_sizes)
    for ti in range(nt):
        for l in range(len(cfg.fit_sizes)):
            fi, fo = fw[l], fw[l + 1]
            pre = f"fitting_net.{ti}.layers.{l}."
            p[pre + "weight"] = t(rng.normal(0, 1 / np.sqrt(fi), (fi, fo)))
            if l == len(cfg.fit_sizes) - 1:
                p[pre + "bias"] = t(np.full((1, fo), shift[ti]))
            else:
                p[pre + "bias"] = t(rng.normal(0, 0.1, (1, fo)))
                if cfg.fit_resnet_dt and l > 0:
                    p[pre + "resnet_dt"] = t(rng.normal(0.1, 0.001, (1, fo)))
    return p


def load_reference_state_dict(sd) -> Dict[str, torch.Tensor]:
    """Take the network tensors of a reference ``DP`` state dict (or ``jit_dp.pt``)."""
    return {k: v.detach().clone() for k, v in sd.items()
            if k.startswith("embedding_net.") or k.startswith("fitting_net.")}


def calc_stat(cfg: DPConfig, list_neigh: np.ndarray, image_dr: np.ndarray,
              types: np.ndarray):
    """davg / dstd per centre type, tiled over all slots: returns two [ntypes, S*4] arrays.

    Restates ``src/pre_data/dpuni_data_loader.py:422-499`` (``calc_stat``) with ``smooth``
    (``:501-563``): per type, the mean of the radial channel s(r) over every slot of every
    atom (empty slots count as 0) and the standard deviations of the radial and of the
    averaged angular channels, floored at 1e-2."""
    ln = list_neigh.reshape(-1, list_neigh.shape[-1])
    dr = image_dr.reshape(-1, ln.shape[-1], 4)
    r = dr[..., 0]
    mask = ln > 0
    rs = np.where(mask, r, 1.0)
    u = (rs - cfg.Rmin) / (cfg.Rmax - cfg.Rmin)
    vv = np.where(rs < cfg.Rmin, 1.0,
                  np.where(rs < cfg.Rmax, u ** 3 * (-6 * u ** 2 + 15 * u - 10) + 1, 0.0))
    vv = np.where(mask, vv, 0.0)
    Ri = np.stack([vv / rs, vv * dr[..., 1] / rs ** 2, vv * dr[..., 2] / rs ** 2,
                   vv * dr[..., 3] / rs ** 2], axis=-1)
    Ri = np.where(mask[..., None], Ri, 0.0)
    S = ln.shape[-1]
    tmap = np.tile(np.asarray(types), ln.shape[0] // len(types))
    davg = np.zeros((cfg.ntypes, S * 4))
    dstd = np.ones((cfg.ntypes, S * 4))

    def std(s2, s, n):
        if n == 0:
            return 1e-2
        v = np.sqrt(max(s2 / n - (s / n) ** 2, 0.0))
        return max(v, 1e-2)

    for t in range(cfg.ntypes):
        sel = Ri[tmap == t].reshape(-1, 4)
        n = sel.shape[0]
        if n == 0:
            continue
        s = sel.sum(0)
        s2 = (sel * sel).sum(0)
        sa, s2a = float(np.mean(s[1:])), float(np.mean(s2[1:]))
        unit_avg = [s[0] / (n + 1e-15), 0.0, 0.0, 0.0]
        unit_std = [std(s2[0], s[0], n)] + [std(s2a, sa, n)] * 3
        davg[t] = np.tile(unit_avg, S)
        dstd[t] = np.tile(unit_std, S)
    return davg, dstd
