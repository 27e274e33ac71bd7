"""Type-embedding DP (``TypeDP``, src/model/dp_dp_typ_emb.py:44-549) on the GPU.

One embedding net shared by all type pairs takes [s_ij, v(t_j)] - the scaled s of the slot and
the neighbor element's normalised physical-property vector v (``type_vector``,
utils/atom_type_emb_dict.py:143-161) - as its first-layer input (dp_embedding_typ_emb.py:
EmbeddingNet with ``type_feat_num``); the contraction, the per-element fitting nets and the
force / virial path are those of DP.  ``TypeDP`` is ``train.DPTrainModel`` (environment matrix,
fitting nets, forces and virial through this library's operators, second-order differentiable
for training) with that embedding; parameter names follow the reference
(``embedding_net.{E}.layers.{l}``, E = index of the embedding net after an optional type
embedding net).

``fused_model`` evaluates the same model in the fused kernels (every precision form) by
folding v(t_j) into the first layer's bias (``dp_params``).  The property vectors are an
input: ``type_vector`` maps each model element to the list the
reference's ``get_normalized_data_list(atom_type, physical_property)`` gives for it (stored
with a trained model; this package does not carry the element property table).  The
reference's optional type-embedding net (``network_size`` non-empty) is not applied to the
vectors by its own forward (calculate_xyz_scater feeds the raw vectors), so it is not used
here either.
"""
import math
from typing import Dict, Sequence

import torch

from .params import DPConfig
from .train import DPTrainModel


def init_type_params(cfg: DPConfig, nfeat: int, seed: int, emb_index: int = 0,
                     dtype=torch.float64) -> Dict[str, torch.Tensor]:
    """Seeded parameters with the reference's shapes and initial distributions
    (dp_embedding_typ_emb.py:71-88 and the fitting net): embedding widths
    [1 + nfeat] + emb_sizes, one fitting net per element on M2 * emb_sizes[-1] inputs."""
    g = torch.Generator().manual_seed(seed)
    p = {}
    widths = [1 + nfeat] + list(cfg.emb_sizes)
    for l in range(len(cfg.emb_sizes)):
        pre = f"embedding_net.{emb_index}.layers.{l}."
        p[pre + "weight"] = torch.randn(widths[l], widths[l + 1], generator=g,
                                        dtype=torch.float64) / math.sqrt(widths[l] + widths[l + 1])
        p[pre + "bias"] = torch.randn(1, widths[l + 1], generator=g, dtype=torch.float64)
        if cfg.emb_resnet_dt:
            p[pre + "resnet_dt"] = 1 + 0.001 * torch.randn(1, widths[l + 1], generator=g,
                                                           dtype=torch.float64)
    fw = [cfg.M2 * cfg.emb_sizes[-1]] + list(cfg.fit_sizes)
    for t in range(cfg.ntypes):
        for l in range(len(cfg.fit_sizes)):
            pre = f"fitting_net.{t}.layers.{l}."
            p[pre + "weight"] = torch.randn(fw[l], fw[l + 1], generator=g,
                                            dtype=torch.float64) / math.sqrt(fw[l] + fw[l + 1])
            p[pre + "bias"] = torch.randn(1, fw[l + 1], generator=g, dtype=torch.float64)
            if cfg.fit_resnet_dt and 0 < l < len(cfg.fit_sizes) - 1:
                p[pre + "resnet_dt"] = 0.1 + 0.001 * torch.randn(1, fw[l + 1], generator=g,
                                                                 dtype=torch.float64)
    return {k: v.to(dtype) for k, v in p.items()}


def dp_params(cfg: DPConfig, params: Dict[str, torch.Tensor], type_vector: Dict[int, Sequence[float]],
              emb_index: int = None) -> Dict[str, torch.Tensor]:
    """The TypeDP model as per-type-pair embedding nets (DP's parameter names): the shared net
    with input [s, v(t_j)] has the first-layer pre-activation s W0[0] + (b0 + v(t_j) W0[1:]),
    so net (t_i, t_j) is DP's 1 -> 25 layer with weight W0[0] and bias b0 + v(t_j) W0[1:],
    followed by the shared 25 -> 25 layers.  The fused evaluation (``dp.DP``, every precision
    form including the tcgen05 ones) then runs TypeDP unchanged."""
    if emb_index is None:
        emb_index = sorted({int(k.split(".")[1]) for k in params if k.startswith("embedding_net.")})[-1]
    pre = f"embedding_net.{emb_index}.layers."
    W0 = params[pre + "0.weight"].detach().to(torch.float64).cpu()
    b0 = params.get(pre + "0.bias")
    b0 = torch.zeros(W0.shape[1], dtype=torch.float64) if b0 is None else \
        b0.detach().to(torch.float64).cpu().reshape(-1)
    out = {k: v for k, v in params.items() if k.startswith("fitting_net.")}
    T = cfg.ntypes
    for ti in range(T):
        for tj in range(T):
            k = ti * T + tj
            v = torch.tensor(list(type_vector[cfg.atom_type[tj]]), dtype=torch.float64)
            q = f"embedding_net.{k}.layers."
            out[q + "0.weight"] = W0[0:1].clone()
            out[q + "0.bias"] = (b0 + v @ W0[1:]).reshape(1, -1)
            for l in (1, 2):
                for name in ("weight", "bias", "resnet_dt"):
                    src = params.get(pre + f"{l}.{name}")
                    if src is not None:
                        out[q + f"{l}.{name}"] = src.detach().to(torch.float64).cpu()
    return out


def fused_model(cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
                type_vector: Dict[int, Sequence[float]], precision: str = "float64",
                device="cuda", emb_index: int = None):
    """TypeDP in the fused evaluation (``dp.DP`` on ``dp_params``)."""
    from .dp import DP
    return DP(cfg, dp_params(cfg, params, type_vector, emb_index), davg, dstd,
              precision=precision, device=device)


class TypeDP(DPTrainModel):
    def __init__(self, cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
                 type_vector: Dict[int, Sequence[float]], emb_index: int = None,
                 dtype=torch.float64, device="cuda"):
        super().__init__(cfg, params, davg, dstd, dtype=dtype, device=device)
        vec = torch.tensor([list(type_vector[z]) for z in cfg.atom_type], dtype=dtype,
                           device=device)
        self.register_buffer("type_vec", vec)
        if emb_index is None:
            idx = sorted({int(k.split(".")[1]) for k in params if k.startswith("embedding_net.")})
            emb_index = idx[-1]
        self.emb_index = emb_index

    def _emb(self, k: int, s: torch.Tensor) -> torch.Tensor:
        # calculate_xyz_scater (dp_dp_typ_emb.py:360-375): [s, v(t_j)] -> the shared net
        tj = k % self.cfg.ntypes
        v = self.type_vec[tj].expand(*s.shape[:-1], self.type_vec.shape[1])
        x = torch.cat((s, v), dim=-1)
        widths = [x.shape[-1]] + list(self.cfg.emb_sizes)
        for l in range(len(self.cfg.emb_sizes)):
            pre = f"embedding_net.{self.emb_index}.layers.{l}."
            h = x @ self.param(pre + "weight")
            b = self.param(pre + "bias")
            h = torch.tanh(h + b if b is not None else h)
            dt = self.param(pre + "resnet_dt")
            if widths[l + 1] == widths[l]:
                x = (h * dt if dt is not None else h) + x
            elif widths[l + 1] == 2 * widths[l]:
                x = torch.cat((x, x), dim=-1) + (h * dt if dt is not None else h)
            else:
                x = h
        return x
