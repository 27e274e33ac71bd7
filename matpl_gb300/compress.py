"""Compressed DP: the embedding nets replaced by piecewise-polynomial tables, the model MatPL's
``compress`` command writes (src/user/ckpt_compress.py) and ``DP.forward`` evaluates through
``calc_compress_polynomial`` and the ``calculateCompress`` op (src/model/dp_dp.py:572-601,
CalcOps.cpp:331-383).

* ``build_table`` restates the table builder: the grid of the normalised s from
  ``set_sij_range`` (:348-377; step dx up to the largest trained s, then 10 dx up to ten times
  it) and per type pair and embedding output the Hermite coefficients of each grid interval
  from G, dG/ds (order 3, ``dp_model_compress_3order``, :110-150) and d2G/ds2 (order 5,
  ``dp_model_compress_5order``, :152-227), derivatives by autograd through the nets.
* ``fused_model`` runs the table inside the fused FP32 / FP64 evaluation kernels (the
  production path); ``CompressedDP`` is the reference's structure on this library's operators
  (``train.DPTrainModel``: environment matrix, contraction, fitting nets, forces / virial) with
  the embedding taken from the table:
  the interval index and offset of ``calc_compress_polynomial`` (including its float32 grid
  point and the coarse-region index it uses as it is) and the polynomial from
  ``ops.calculateCompress`` (csrc/compress.cu), differentiable in s for the forces.
"""
from typing import Dict

import numpy as np
import torch

from . import ops
from .params import DPConfig
from .train import DPTrainModel


def sij_range(davg, dstd, sij_max: float, dx: float):
    """set_sij_range (ckpt_compress.py:348-377) -> (grid [L], scal_min, scal_max, sij_out_max,
    len_sij, len_out_max); davg / dstd [ntypes, ...] with the radial unit in column 0."""
    davg = np.asarray(davg)
    dstd = np.asarray(dstd)
    scal_max, scal_min = 0, 0
    for i in range(davg.shape[0]):
        smax = (sij_max - davg[i, 0]) / dstd[i, 0]
        scal_max = smax if smax > scal_max else scal_max
        smin = (0 - davg[i, 0]) / dstd[i, 0]
        scal_min = smin if smin < scal_min else scal_min
    grid = []
    s = scal_min
    while s < scal_max:
        grid.append(s)
        s += dx
    len_sij = len(grid)
    sij_out_max = scal_max * 10
    len_out = 0
    while s < sij_out_max:
        grid.append(s)
        s += dx * 10
        len_out += 1
    return np.array(grid), scal_min, scal_max, sij_out_max, len_sij, len_out


def _hermite(y, y1, y2, dx, order):
    """Coefficients (highest power first) of each interval [k, k+1] from values and
    derivatives at its ends (ckpt_compress.py:130-138 for order 3, :187-204 for order 5)."""
    a, b = y[:-1], y[1:]
    a1, b1 = y1[:-1], y1[1:]
    if order == 3:
        am = 1 / dx ** 3 * ((b1 + a1) * dx - 2 * (b - a))
        bm = 1 / dx ** 2 * (-(b1 + 2 * a1) * dx + 3 * (b - a))
        return torch.stack([am, bm, a1, a], -1)
    a2, b2 = y2[:-1], y2[1:]
    am = 1 / (2 * dx ** 5) * (12 * (b - a) - 6 * (b1 + a1) * dx + (b2 - a2) * dx ** 2)
    bm = 1 / (2 * dx ** 4) * (-30 * (b - a) + (14 * b1 + 16 * a1) * dx
                              + (3 * a2 - 2 * b2) * dx ** 2)
    cm = 1 / (2 * dx ** 3) * (20 * (b - a) - (8 * b1 + 12 * a1) * dx - (3 * a2 - b2) * dx ** 2)
    return torch.stack([am, bm, cm, 0.5 * a2, a1, a], -1)


def build_table(cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd, sij_max: float,
                dx: float = 0.01, order: int = 5, device="cpu",
                reference_dx_growth: bool = True) -> Dict:
    """The ``compress`` dict of ckpt_compress.compress_force_field (:37-85): table
    [ntypes^2, rows, width, order + 1] and the grid parameters.

    The reference's builders multiply their interval width by 10 for the coarse region inside
    the loop over type pairs without resetting it (ckpt_compress.py:118-124, 161-172), so type
    pair p gets coefficients for widths 10^p dx (fine) and 10^(p+1) dx (coarse) on the same
    grid.  ``reference_dx_growth`` (default) reproduces that, as the tables of the reference's
    compressed checkpoints hold it; False gives every pair the widths of its grid."""
    if order not in (3, 5):
        raise ValueError("compress order 3 or 5")
    model = DPTrainModel(cfg, params, davg, dstd, dtype=torch.float64, device=device)
    grid, smin, smax, out_max, len_sij, len_out = sij_range(davg, dstd, sij_max, dx)
    sij = torch.tensor(grid, dtype=torch.float64, device=device).unsqueeze(-1)
    tabs = []
    width = dx
    for t0 in range(cfg.ntypes):
        for t1 in range(cfg.ntypes):
            k = t0 * cfg.ntypes + t1
            fine = width if reference_dx_growth else dx
            coarse = 10 * fine
            if reference_dx_growth:
                width = coarse
            rows = []
            for part, h in ((sij[:len_sij + 1], fine), (sij[len_sij:], coarse)):
                s = part.detach().clone().requires_grad_()
                y = model._emb(k, s)
                d1, d2 = [], []
                for m in range(y.shape[-1]):
                    g1 = torch.autograd.grad(y[:, m].sum(), s, create_graph=order == 5,
                                             retain_graph=True)[0]
                    d1.append(g1[:, 0])
                    if order == 5:
                        d2.append(torch.autograd.grad(g1.sum(), s, retain_graph=True)[0][:, 0])
                Y = y.detach()
                D1 = torch.stack(d1, -1).detach()
                D2 = torch.stack(d2, -1).detach() if order == 5 else None
                rows.append(_hermite(Y, D1, D2, h, order))
            tabs.append(torch.cat(rows, 0))
    table = torch.stack(tabs).cpu().numpy()
    return {"table": table, "dx": dx, "order": order, "sij_min": smin, "sij_max": smax,
            "sij_out_max": out_max, "sij_len": len_sij, "sij_out_len": len_out,
            "davg": np.asarray(davg)[:, 0], "dstd": np.asarray(dstd)[:, 0]}


def fused_model(cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd, compress: Dict,
                precision: str = "float64", device="cuda"):
    """The compressed model in the fused evaluation (``matpl_dp_eval`` with the table in
    ``matpl_dp_model.ctable``: environment row, table polynomial, descriptor, fitting nets,
    adjoint and force / virial scatter in the FP32 / FP64 kernels, no per-slot tensors)."""
    from .dp import DP
    return DP(cfg, params, davg, dstd, precision=precision, device=device, compress=compress)


class CompressedDP(DPTrainModel):
    """DP with tabulated embeddings (inference: E, Ei, forces, virial)."""

    def __init__(self, cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
                 compress: Dict, dtype=torch.float64, device="cuda"):
        super().__init__(cfg, params, davg, dstd, dtype=dtype, device=device)
        tab = torch.as_tensor(np.asarray(compress["table"]), dtype=dtype, device=device)
        self.tab_rows = tab.shape[1]
        self.register_buffer("table", tab.reshape(tab.shape[0] * tab.shape[1], tab.shape[2],
                                                  tab.shape[3]).contiguous())
        self.dx = float(compress["dx"])
        self.sij_min = float(compress["sij_min"])
        self.sij_max = float(compress["sij_max"])

    def _emb(self, k: int, s: torch.Tensor) -> torch.Tensor:
        # calc_compress_polynomial (dp_dp.py:572-601) for one type pair
        shape = s.shape[:-1]
        sij = s.reshape(-1)
        mask = sij < self.sij_max
        x = torch.where(mask, (sij - self.sij_min) / self.dx,
                        (sij - self.sij_max) / (10 * self.dx))
        idx = x.detach().to(torch.long)                        # truncation, like .type(long)
        xk = torch.where(mask, idx * self.dx + self.sij_min,   # float32 arithmetic, as in the
                         self.sij_max + idx * self.dx * 10)    # reference's float32 grid point
        f2 = (sij - xk.to(torch.float32).to(sij.dtype)).unsqueeze(-1)
        coeff = self.table[idx + k * self.tab_rows]
        G = ops.calculateCompress(f2, coeff)[0]
        return G.reshape(*shape, G.shape[-1])
