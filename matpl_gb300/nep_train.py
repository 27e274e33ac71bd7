"""Trainable NEP on GB300: ``nep_net.NEP.forward``'s CUDA branch (src/model/nep_net.py:293-438,
503-648) on this library's operators.

``NEPTrain`` holds the parameters under the reference's names (``c_param_2``, ``c_param_3``,
``fitting_net.{t}.layers.{0,1}.weight / bias``, buffer ``q_scaler``), so reference checkpoints
load unchanged, and its forward takes the lists of ``calculate_neighbor``.  The descriptor runs
``calculateNepFeat`` / ``calculateNepMbFeat`` (csrc/nep_train.cu: the forward, backward and
second backward that the force loss needs, and the coefficient gradient); forces and virial run
``nep_force_virial``, the kernel form of calculate_Ri + calculateNepForce + calculateNepVirial
that reads the rows (r, x, y, z) and forms d(r, x, y, z)/d(x, y, z) in registers.  With
``create_graph`` forces, ``loss.backward()`` of an energy + force + virial loss reaches every
parameter exactly like the reference's training step (nep_trainer.py), through the hand-written
second derivatives instead of autograd over the descriptor.  The per-element FittingNet (one
tanh layer, nep_fitting.py:136-160) stays in torch, all elements in one product
(``calculate_Ei``).
"""
from typing import Dict, Optional

import torch

from . import nep_ops
from . import splitk
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
    mask = (Ri[:, :, 0:1].abs() > 1e-5).to(Ri.dtype)
    safe = torch.where(mask > 0, Ri[:, :, 0:1], torch.ones_like(mask))
    eye = torch.eye(3, dtype=Ri.dtype, device=Ri.device)
    return torch.cat(((Ri[:, :, 1:] / safe * mask).unsqueeze(2), eye * mask.unsqueeze(-1)), 2)


def _image_sum(x: torch.Tensor, counts) -> torch.Tensor:
    """Per-image sums [B, ...] of per-atom rows x [N, ...] (frames contiguous, sizes
    ``counts``): one reduction when the frames have one size (batches of one composition),
    else an index_add over the atoms' image index."""
    B = len(counts)
    if B == 1:
        return x.sum(0, keepdim=True)
    if all(c == counts[0] for c in counts):
        return x.reshape((B, counts[0]) + tuple(x.shape[1:])).sum(1)
    img = nep_ops._image_index(tuple(counts), x.device)
    return torch.zeros((B,) + tuple(x.shape[1:]), dtype=x.dtype,
                       device=x.device).index_add(0, img, x)


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
        H = p["fitting_net.0.layers.0.weight"].shape[1]
        blocks = torch.eye(cfg.ntypes, dtype=dtype, device=dev).repeat_interleave(H, 0)
        self.register_buffer("fit_blocks", blocks, persistent=False)              # [T*H, T]

    def type_index(self, type_map: torch.Tensor) -> torch.Tensor:
        """[N, T] one-hot centre type of every atom (no host synchronisation); ``forward`` makes
        it when none is passed."""
        tm = type_map.reshape(-1, 1).long()
        return (tm == torch.arange(self.cfg.ntypes, device=tm.device)).to(self.q_scaler.dtype)

    def calculate_Ei(self, type_map: torch.Tensor, feats: torch.Tensor,
                     type_index: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Ei [N]: each atom through its element's FittingNet (nep_net.py:470-501).  All T nets
        run on all atoms as one [N, F] x [F, T*H] product and each atom keeps its own net's
        output through the one-hot type: a few well-shaped launches (and their backward and
        double backward) in place of per-element gathers, small GEMMs and scatters; the other
        elements' outputs are multiplied by zero, so every parameter's gradient is that of the
        per-element evaluation."""
        onehot = type_index if type_index is not None else self.type_index(type_map)
        nets = self.fitting_net
        W0 = torch.cat([net.layers[0].weight for net in nets], 1)                 # [F, T*H]
        b0 = torch.cat([net.layers[0].bias.reshape(-1) for net in nets])          # [T*H]
        # output layers as one block-diagonal [T*H, T] matrix
        W1 = torch.cat([net.layers[1].weight for net in nets], 0) * self.fit_blocks
        b1 = torch.cat([net.layers[1].bias.reshape(-1) for net in nets])          # [T]
        h = torch.tanh(splitk.add_row(splitk.mm(feats, W0), b0))
        y = splitk.add_row(splitk.mm(h, W1), b1)                                  # [N, T]
        return (y * onehot).sum(-1)

    def forward(self, NN_radial, NL_radial, Ri_radial, NN_angular, NL_angular, Ri_angular,
                num_atom, atom_type_map, Egroup_weight: Optional[torch.Tensor] = None,
                divider: Optional[torch.Tensor] = None, is_calc_f: bool = True,
                type_index: Optional[torch.Tensor] = None):
        cfg = self.cfg
        dt = self.q_scaler.dtype
        tm = atom_type_map.reshape(-1).long()
        Ri = Ri_radial.to(dt).detach()
        Ra = Ri_angular.to(dt).detach()
        N = tm.shape[0]
        # descriptor parts: (coefficients, rows, list, angular, cutoff, features)
        parts = []
        if cfg.train_2b:
            parts.append((self.c_param_2, Ri, NL_radial, False, cfg.cutoff[0], cfg.two_feat_num))
        if cfg.l_max[0] > 0:
            parts.append((self.c_param_3, Ra, NL_angular, True, cfg.cutoff[1],
                          cfg.multi_feat_num))
        feats = []
        for c, R, NL, ang, rc, nf in parts:
            buf = torch.zeros(N, nf, dtype=dt, device=Ri.device)
            if ang:
                feats.append(nep_ops.calculateNepMbFeat(c, R, NL, tm, buf, cfg.two_feat_num,
                                                        *cfg.l_max, rc)[0])
            else:
                feats.append(nep_ops.calculateNepFeat(c, R, NL, tm, buf, rc,
                                                      cfg.multi_feat_num)[0])
        feats = torch.cat(feats, -1)
        Ei = self.calculate_Ei(tm, self.q_scaler * feats, type_index)
        counts = tuple(int(c) for c in num_atom.reshape(-1).tolist())
        zbl = None
        if cfg.zbl is not None:
            # ZBL term (nep_net.py:399-408, 916-991): parameter-free, so its energy, forces and
            # virial enter as constants
            zbl = (torch.zeros(N, dtype=dt, device=Ri.device),
                   torch.zeros(N, 3, dtype=dt, device=Ri.device),
                   torch.zeros(len(counts), 9, dtype=torch.float64, device=Ri.device))
            nep_ops.nep_zbl(cfg.zbl, cfg.atom_type, NL_angular, Ra, tm, counts, zbl[0], None,
                            zbl[1], zbl[2])
            Ei = Ei + zbl[0]
        Etot = _image_sum(Ei, counts).unsqueeze(-1)
        Egroup = None
        if Egroup_weight is not None and divider is not None:
            Egroup = torch.divide(torch.matmul(Egroup_weight, Ei.unsqueeze(-1)).squeeze(-1), divider)
        if not is_calc_f:
            return Etot, Ei, None, Egroup, None
        # dE/dd12 of each list (nep_net.py:603-611): dEtot/dq through the fitting nets, then
        # G . dq/dd12 by the descriptor's backward mode alone (no coefficient table), kept
        # differentiable in G and the coefficients for the force and virial loss
        G = torch.autograd.grad(Etot.sum(), feats, create_graph=True)[0]
        Force = torch.zeros(N, 3, dtype=dt, device=Ri.device)
        Virial = torch.zeros(len(counts), 9, dtype=dt, device=Ri.device)
        off = 0
        for c, R, NL, ang, rc, nf in parts:         # nep_net.py:612-631
            dE = nep_ops.nep_feat_d12(c, G[:, off:off + nf], R, NL, tm, ang, rc,
                                      *(cfg.l_max if ang else (0, 0, 0)))
            off += nf
            # calculateNepForce + calculateNepVirial of the list with calculate_Ri formed in the
            # kernel (one pass over the slots, no [N, NN, 4, 3] array)
            F_l, V_l = nep_ops.nep_force_virial(NL, dE, R, counts)
            Force = Force + F_l
            Virial = Virial + V_l
        if zbl is not None:          # physical force / virial of the ZBL term: -(op convention)
            Force = Force - zbl[1]
            Virial = Virial - zbl[2].to(dt)
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
        with torch.cuda.graph(g, stream=side):   # the warm-up's workspaces are reused
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

