"""Force-loss training step of DP se_e2_a on the GPU (the path of ``dp_trainer.train``,
``src/PWMLFF/dp_mods/dp_trainer.py:119-275``, with the model of ``src/model/dp_dp.py`` on CUDA).

The model keeps the reference's parameter names (``embedding_net.{k}.layers.{l}.weight`` ...)
as ``torch.nn.Parameter``s.  One evaluation is

* environment matrix Ri, Ri_d from ``matpl_gb300.ops.env_mat`` (this library's kernel);
* embedding / fitting nets and dE/dRi by autograd with ``create_graph=True`` (dp_dp.py:429);
* forces and virial from ``ops.calculateForce`` / ``ops.calculateVirial`` (this library's
  kernels, differentiable in dE: their backward kernels feed the second-order gradient);

and ``train_step`` applies the reference loss (dp_trainer.py:172-272 with ``dp_loss``'s
prefactors, ``src/loss/dploss.py:18-66``) and the optimizer.  Configurations are evaluated one
composition cluster at a time, as the reference does (``_classify_batchs``, dp_trainer.py:536).
"""
from typing import Dict, List, Optional, Sequence

import torch

from . import ops
from .params import DPConfig


class DPTrainModel(torch.nn.Module):
    def __init__(self, cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
                 dtype=torch.float64, device="cuda"):
        super().__init__()
        self.cfg = cfg
        self.dtype = dtype
        self.names = sorted(params.keys())
        self.p = torch.nn.ParameterDict({k.replace(".", "__"): torch.nn.Parameter(
            params[k].detach().to(device=device, dtype=dtype).clone()) for k in self.names})
        self.register_buffer("davg", torch.as_tensor(davg).to(device=device, dtype=dtype))
        self.register_buffer("dstd", torch.as_tensor(dstd).to(device=device, dtype=dtype))

    def param(self, name: str) -> Optional[torch.Tensor]:
        return self.p[name.replace(".", "__")] if name.replace(".", "__") in self.p else None

    def _emb(self, k: int, s: torch.Tensor) -> torch.Tensor:
        widths = [1] + list(self.cfg.emb_sizes)
        x = s
        for l in range(len(self.cfg.emb_sizes)):
            pre = f"embedding_net.{k}.layers.{l}."
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

    def _fit(self, t: int, x: torch.Tensor) -> torch.Tensor:
        nl = len(self.cfg.fit_sizes)
        for l in range(nl - 1):
            pre = f"fitting_net.{t}.layers.{l}."
            h = x @ self.param(pre + "weight")
            b = self.param(pre + "bias")
            h = torch.tanh(h + b if b is not None else h)
            if l == 0:
                x = h
            else:
                dt = self.param(pre + "resnet_dt")
                x = (h * dt if dt is not None else h) + x
        pre = f"fitting_net.{t}.layers.{nl - 1}."
        y = x @ self.param(pre + "weight")
        b = self.param(pre + "bias")
        return y + b if b is not None else y

    def forward(self, list_neigh, Imagetype_map, atom_type, ImageDR, nghost: int = 0):
        """(Etot [B,1], Ei [B,N] type-grouped, Force [B,N+nghost,3], Virial [B,9]), all
        differentiable w.r.t. the parameters (forces through the second-order graph)."""
        cfg = self.cfg
        B, N, S = list_neigh.shape
        m = cfg.maxNeighborNum
        present = [cfg.atom_type.index(int(a)) for a in atom_type if int(a) in cfg.atom_type]
        T = len(present)
        idr = ImageDR.to(self.dtype)
        Ri, Ri_d = ops.env_mat(idr, Imagetype_map, self.davg, self.dstd, cfg.Rmin, cfg.Rmax)
        Ri = Ri.detach().requires_grad_()
        tmap = Imagetype_map.long()
        Ei_blocks = []
        for ti in present:
            idx = torch.nonzero(tmap == ti).flatten()
            if idx.numel() == 0:
                continue
            A = None
            for tj in present:
                blk = Ri[:, idx, tj * m:(tj + 1) * m, :]
                G = self._emb(ti * cfg.ntypes + tj, blk[..., 0:1])
                c = blk.transpose(-2, -1) @ G
                A = c if A is None else A + c
            A = A / (m * T)
            D = A.transpose(-2, -1) @ A[..., :cfg.M2]
            Ei_blocks.append(self._fit(ti, D.reshape(B, idx.numel(), -1)))
        Ei = torch.cat(Ei_blocks, dim=1)
        Etot = Ei.sum(1)
        dE = torch.autograd.grad([Etot], [Ri], grad_outputs=[torch.ones_like(Etot)],
                                 retain_graph=True, create_graph=True)[0]
        Rd = Ri_d.reshape(B, N, 4 * S, 3)
        dEv = dE.reshape(B, N, 1, 4 * S)
        Fc = -(dEv @ Rd).squeeze(-2)
        nl0 = (list_neigh.to(torch.int32) - 1).unsqueeze(2)
        Force = ops.calculateForce(nl0, dEv, Rd, Fc, nghost)[0]
        Virial = ops.calculateVirial(nl0, dEv, idr[..., 1:].contiguous(), Rd, nghost)[0]
        return Etot, Ei.squeeze(-1), Force, Virial


def dp_loss_prefactors(real_lr: float, start_lr: float = 0.001, pre_f=(1000.0, 1.0),
                       pre_e=(0.02, 1.0)):
    """``dp_loss`` prefactor schedule (dploss.py:34-44): limit + (start - limit) * lr/start_lr."""
    f = pre_f[1] + (pre_f[0] - pre_f[1]) * real_lr / start_lr
    e = pre_e[1] + (pre_e[0] - pre_e[1]) * real_lr / start_lr
    return f, e


def loss_fn(model: DPTrainModel, batch: dict, w_f: float = 1.0, w_e: float = 1.0,
            per_atom_energy: bool = False):
    """Force-loss objective of one composition cluster: w_e * MSE(Etot) [/ natoms when
    ``per_atom_energy``, as dp_loss does] + w_f * MSE(F)."""
    Etot, Ei, F, V = model(batch["list_neigh"], batch["type_map"], batch["atom_type"],
                           batch["ImageDR"], 0)
    n = batch["list_neigh"].shape[1]
    le = torch.nn.functional.mse_loss(Etot, batch["Etot"].to(Etot.dtype))
    lf = torch.nn.functional.mse_loss(F[:, :n], batch["Force"].to(F.dtype))
    if per_atom_energy:
        le = le / n
    return w_e * le + w_f * lf, le, lf


def train_step(model: DPTrainModel, batches: Sequence[dict], optimizer: torch.optim.Optimizer,
               w_f: float = 1.0, w_e: float = 1.0):
    """One optimizer step per composition cluster, like the reference's inner loop
    (dp_trainer.py:119-275).  Returns the summed loss."""
    total = 0.0
    for b in batches:
        optimizer.zero_grad(set_to_none=True)
        loss, _, _ = loss_fn(model, b, w_f, w_e)
        loss.backward()
        optimizer.step()
        total += float(loss.detach())
    return total
