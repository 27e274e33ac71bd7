"""Trainable NEP on GB300: ``nep_net.NEP.forward``'s CUDA branch (src/model/nep_net.py:293-438,
503-648) on this library's operators.

``NEPTrain`` holds the parameters under the reference's names (``c_param_2``, ``c_param_3``,
``fitting_net.{t}.layers.{0,1}.weight / bias``, buffer ``q_scaler``), so reference checkpoints
load unchanged, and its forward takes the lists of ``calculate_neighbor``.  The descriptor runs
``calculateNepFeat`` / ``calculateNepMbFeat`` (csrc/nep_train.cu: the forward, backward and
second backward that the force loss needs), forces and virial ``calculateNepForce`` /
``calculateNepVirial``; with ``create_graph`` forces, ``loss.backward()`` of an energy + force +
virial loss reaches every parameter exactly like the reference's training step
(nep_trainer.py), through the hand-written second derivatives instead of autograd over the
descriptor.  The per-element FittingNet (one tanh layer, nep_fitting.py:136-160) stays in
torch: it is a few small GEMMs per element.
"""
from typing import Dict, List, Optional

import torch

from . import nep_ops
from .nep import NepConfig


class _Layer(torch.nn.Module):
    def __init__(self, w: torch.Tensor, b: torch.Tensor):
        super().__init__()
        self.weight = torch.nn.Parameter(w.clone())
        self.bias = torch.nn.Parameter(b.clone())


class _FittingNet(torch.nn.Module):
    def __init__(self, layers):
        super().__init__()
        self.layers = torch.nn.ModuleList(layers)

    def forward(self, x):       # nep_fitting.py:136-160 with one hidden layer
        h = torch.tanh(torch.matmul(x, self.layers[0].weight) + self.layers[0].bias)
        return torch.matmul(h, self.layers[1].weight) + self.layers[1].bias


def calculate_Ri(Ri: torch.Tensor) -> torch.Tensor:
    """[N, NN, 4, 3] d(r, x, y, z)/d(x, y, z) of the non-empty slots (nep_net.py:440-468)."""
    N, NN = Ri.shape[:2]
    mask = (Ri[:, :, 0].abs() > 1e-5).to(Ri.dtype)
    safe = torch.where(mask > 0, Ri[:, :, 0], torch.ones_like(Ri[:, :, 0]))
    d = torch.zeros(N, NN, 4, 3, dtype=Ri.dtype, device=Ri.device)
    for a in range(3):
        d[:, :, 0, a] = Ri[:, :, 1 + a] / safe * mask
        d[:, :, 1 + a, a] = mask
    return d


class NEPTrain(torch.nn.Module):
    def __init__(self, cfg: NepConfig, params: Dict[str, torch.Tensor], dtype=torch.float64,
                 device="cuda"):
        super().__init__()
        self.cfg = cfg
        dev = torch.device(device)
        p = {k: v.to(device=dev, dtype=dtype) for k, v in params.items()}
        if cfg.train_2b:
            self.c_param_2 = torch.nn.Parameter(p["c_param_2"].clone())
        if cfg.l_max[0] > 0:
            self.c_param_3 = torch.nn.Parameter(p["c_param_3"].clone())
        self.fitting_net = torch.nn.ModuleList()
        for t in range(cfg.ntypes):
            pre = f"fitting_net.{t}.layers."
            self.fitting_net.append(_FittingNet([_Layer(p[pre + "0.weight"], p[pre + "0.bias"]),
                                                 _Layer(p[pre + "1.weight"], p[pre + "1.bias"])]))
        self.register_buffer("q_scaler", p["q_scaler"].clone())

    def type_index(self, type_map: torch.Tensor) -> List[torch.Tensor]:
        """Atom indices of every element (one device sync); pass it to ``forward`` to keep the
        step free of host synchronisation (CUDA-graph capture)."""
        tm = type_map.reshape(-1).long()
        return [torch.nonzero(tm == t).flatten() for t in range(self.cfg.ntypes)]

    def calculate_Ei(self, type_map: torch.Tensor, feats: torch.Tensor,
                     type_index: Optional[List[torch.Tensor]] = None) -> torch.Tensor:
        Ei = torch.zeros(type_map.shape[0], dtype=feats.dtype, device=feats.device)
        idxs = type_index if type_index is not None else self.type_index(type_map)
        for idx, net in zip(idxs, self.fitting_net):     # nep_net.py:470-501
            if idx.numel() == 0:
                continue
            Ei = Ei.index_put((idx,), net(feats[idx]).squeeze(-1))
        return Ei

    def forward(self, NN_radial, NL_radial, Ri_radial, NN_angular, NL_angular, Ri_angular,
                num_atom, atom_type_map, Egroup_weight: Optional[torch.Tensor] = None,
                divider: Optional[torch.Tensor] = None, is_calc_f: bool = True,
                type_index: Optional[List[torch.Tensor]] = None):
        cfg = self.cfg
        dt = self.q_scaler.dtype
        tm = atom_type_map.reshape(-1).long()
        Ri = Ri_radial.to(dt).detach().clone().requires_grad_()
        Ra = Ri_angular.to(dt).detach().clone().requires_grad_()
        N = tm.shape[0]
        feats = []
        if cfg.train_2b:
            feats.append(nep_ops.calculateNepFeat(
                self.c_param_2, Ri, NL_radial, tm, torch.zeros(N, cfg.two_feat_num, dtype=dt,
                                                               device=Ri.device),
                cfg.cutoff[0], cfg.multi_feat_num)[0])
        if cfg.l_max[0] > 0:
            feats.append(nep_ops.calculateNepMbFeat(
                self.c_param_3, Ra, NL_angular, tm, torch.zeros(N, cfg.multi_feat_num, dtype=dt,
                                                                device=Ri.device),
                cfg.two_feat_num, *cfg.l_max, cfg.cutoff[1])[0])
        feats = torch.cat(feats, -1)
        Ei = self.calculate_Ei(tm, self.q_scaler * feats, type_index)
        counts = num_atom.reshape(-1).tolist()
        Etot = torch.stack([e.sum() for e in Ei.split(counts)]).unsqueeze(-1)
        Egroup = None
        if Egroup_weight is not None and divider is not None:
            Egroup = torch.divide(torch.matmul(Egroup_weight, Ei.unsqueeze(-1)).squeeze(-1), divider)
        if not is_calc_f:
            return Etot, Ei, None, Egroup, None
        leaves = ([(Ri, NL_radial)] if cfg.train_2b else []) + \
                 ([(Ra, NL_angular)] if cfg.l_max[0] > 0 else [])
        grads = torch.autograd.grad([Etot], [r for r, _ in leaves],
                                    grad_outputs=[torch.ones_like(Etot)], retain_graph=True,
                                    create_graph=True, allow_unused=True)
        Force = torch.zeros(N, 3, dtype=dt, device=Ri.device)
        Virial = torch.zeros(len(counts), 9, dtype=dt, device=Ri.device)
        na = num_atom.reshape(-1)
        for dE, (R, NL) in zip(grads, leaves):        # nep_net.py:612-631
            if dE is None:
                continue
            Rd = calculate_Ri(R.detach())
            f0 = -torch.matmul(dE.reshape(N, 1, -1), Rd.reshape(N, -1, 3)).squeeze(-2)
            Force = Force + nep_ops.calculateNepForce(NL, dE, Rd, f0)[0]
            Virial = Virial + nep_ops.calculateNepVirial(NL, dE, R.detach()[:, :, 1:], Rd, na)[0]
        return Etot, Ei, -Force, Egroup, -Virial


class GraphedNepTrainer:
    """One NEP training step - NEPTrain forward with create_graph forces, the loss
    w_e * MSE(E / atom) + w_f * MSE(F) + w_v * MSE(V / atom), backward through the hand-written
    descriptor derivatives, optimizer update - captured once per batch shape in a CUDA graph and
    replayed: a step costs one graph launch plus copying the batch into the graph's static
    buffers.  ``num_atom`` is a host tensor (frame sizes are part of the shape key); the
    optimizer keeps its state on the device (Adam / AdamW with capturable=True, or SGD).  The
    descriptor kernels' error word is checked by ``check_errors()``, not per step."""

    KEYS = ("NN_r", "NL_r", "Ri_r", "NN_a", "NL_a", "Ri_a", "type_map", "Etot", "Force", "Virial")

    def __init__(self, model: NEPTrain, optimizer: torch.optim.Optimizer, w_e: float = 1.0,
                 w_f: float = 1.0, w_v: float = 0.0, warmup: int = 3):
        self.model, self.opt = model, optimizer
        self.w = (w_e, w_f, w_v)
        self.warmup = warmup
        self.graphs = {}

    def loss(self, b, type_index=None):
        Etot, _, F, _, V = self.model(b["NN_r"], b["NL_r"], b["Ri_r"], b["NN_a"], b["NL_a"],
                                      b["Ri_a"], b["num_atom"], b["type_map"],
                                      type_index=type_index)
        per = b["per_atom"]
        w_e, w_f, w_v = self.w
        loss = w_e * ((Etot.reshape(-1) - b["Etot"]) / per).pow(2).mean() \
            + w_f * (F - b["Force"]).pow(2).mean()
        if w_v:
            loss = loss + w_v * ((V - b["Virial"]) / per.unsqueeze(-1)).pow(2).mean()
        return loss

    def _capture(self, batch):
        dt = self.model.q_scaler.dtype
        static = {k: batch[k].clone() for k in self.KEYS}
        for k in ("Ri_r", "Ri_a", "Etot", "Force", "Virial"):
            static[k] = static[k].to(dt)
        static["num_atom"] = batch["num_atom"].detach().cpu().reshape(-1)
        static["per_atom"] = static["num_atom"].to(device=static["Etot"].device, dtype=dt)
        tindex = self.model.type_index(static["type_map"])
        nep_ops.set_check_errors(False)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(self.warmup):         # allocator, image index, kernel attributes
                self.opt.zero_grad(set_to_none=True)
                self.loss(static, tindex).backward()
                self.opt.step()
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        self.opt.zero_grad(set_to_none=True)
        with torch.cuda.graph(g):
            loss = self.loss(static, tindex)
            loss.backward()
            self.opt.step()
        return g, static, loss

    def step(self, batch) -> torch.Tensor:
        key = tuple(tuple(batch[k].shape) for k in self.KEYS) + \
            (tuple(batch["num_atom"].reshape(-1).tolist()),)
        if key not in self.graphs:
            self.graphs[key] = self._capture(batch)
        g, static, loss = self.graphs[key]
        for k in self.KEYS:
            if batch[k].data_ptr() != static[k].data_ptr():
                static[k].copy_(batch[k], non_blocking=True)
        g.replay()
        return loss

    def check_errors(self):
        nep_ops.check_errors()

