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

from . import ops, splitk
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


def _atom_order_energies(model: DPTrainModel, Ei: torch.Tensor, type_map: torch.Tensor,
                         atom_type) -> torch.Tensor:
    """Ei of DPTrainModel.forward (type-grouped, dp_dp.py:339) back in atom order."""
    cfg = model.cfg
    present = [cfg.atom_type.index(int(a)) for a in atom_type if int(a) in cfg.atom_type]
    tl = type_map.long().reshape(-1)
    order = torch.cat([torch.nonzero(tl == ti).flatten() for ti in present])
    return Ei.new_zeros(tl.numel()).index_copy(0, order, Ei.reshape(-1))


def loss_fn(model: DPTrainModel, batch: dict, w_f: float = 1.0, w_e: float = 1.0,
            per_atom_energy: bool = False):
    """Force-loss objective of one composition cluster: w_e * MSE(Etot) [/ natoms when
    ``per_atom_energy``, as dp_loss does] + w_f * MSE(F).  A ragged batch
    (``data.ragged_batch``) takes the MSE over its configurations' energies."""
    Etot, Ei, F, V = model(batch["list_neigh"], batch["type_map"], batch["atom_type"],
                           batch["ImageDR"], 0)
    n = batch["list_neigh"].shape[1]
    if "config_of_atom" in batch:
        from .data import config_energies
        Ei_atom = _atom_order_energies(model, Ei, batch["type_map"], batch["atom_type"])
        Etot = config_energies(Ei_atom, batch["config_of_atom"], batch["Etot"].numel())
    le = torch.nn.functional.mse_loss(Etot, batch["Etot"].to(Etot.dtype).reshape(Etot.shape))
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


# ----------------------------------------------------------------------------------------------
# Fused force-loss gradient: the embedding nets' second-order part runs in this library's
# kernels (matpl_dp_dual_forward / matpl_dp_dual_backward, recomputing activations), the small
# per-atom fitting part in torch.
# ----------------------------------------------------------------------------------------------
import ctypes  # noqa: E402

from . import _lib, dp as _dp  # noqa: E402
from ._lib import check as _check, ptr as _ptr  # noqa: E402


_CONSTS: Dict[tuple, torch.Tensor] = {}


def _const(n: int, fill: float, like: torch.Tensor) -> torch.Tensor:
    """A constant vector (an absent bias or resnet_dt) made once per device and dtype, so that
    a training step spends no fill launch on it."""
    key = (n, fill, like.dtype, like.device)
    v = _CONSTS.get(key)
    if v is None:
        v = _CONSTS[key] = torch.full((n,), fill, dtype=like.dtype, device=like.device)
    return v


def _emb_flat(model: DPTrainModel) -> torch.Tensor:
    """Embedding parameters of every (t_i, t_j) net in the packed order of csrc/dp_layout.cuh,
    built from the model's Parameters with differentiable ops (gradients flow back to them)."""
    E = _dp.E
    parts = []
    for k in range(model.cfg.ntypes ** 2):
        pre = f"embedding_net.{k}.layers."
        for l in range(3):
            w = model.param(pre + f"{l}.weight")
            b = model.param(pre + f"{l}.bias")
            parts.append(w.reshape(-1))
            parts.append(b.reshape(-1) if b is not None else _const(E, 0.0, w))
            if l > 0:
                dt = model.param(pre + f"{l}.resnet_dt")
                parts.append(dt.reshape(-1) if dt is not None else _const(E, 1.0, w))
    return torch.cat(parts)


def _pack_device(model: DPTrainModel) -> torch.Tensor:
    """Full packed parameter buffer (csrc/dp_layout.cuh) on the model's device, no autograd."""
    cfg, F, DIN = model.cfg, _dp.F, _dp.DIN
    with torch.no_grad():
        parts = [_emb_flat(model)]
        for t in range(cfg.ntypes):
            pre = f"fitting_net.{t}.layers."

            def g(name, n, fill):
                v = model.param(pre + name)
                return v.reshape(-1) if v is not None else _const(n, fill, model.davg)
            W0, W1, W2 = g("0.weight", 0, 0), g("1.weight", 0, 0), g("2.weight", 0, 0)
            parts += [W0, g("0.bias", F, 0.0), W1, g("1.bias", F, 0.0), g("1.resnet_dt", F, 1.0),
                      W2, g("2.bias", F, 0.0), g("2.resnet_dt", F, 1.0), g("3.weight", 0, 0),
                      g("3.bias", 1, 0.0), _const(3, 0.0, model.davg),
                      W0.reshape(DIN, F).t().reshape(-1), W1.reshape(F, F).t().reshape(-1),
                      W2.reshape(F, F).t().reshape(-1)]
        return torch.cat(parts).contiguous()


class _EmbedDual(torch.autograd.Function):
    """(A, A_dot) = per-atom descriptor factor over occupied slots and its tangent along the
    force / virial seed (matpl_dp_dual_forward); the backward is matpl_dp_dual_backward."""

    @staticmethod
    @_lib.on_device
    def forward(ctx, emb_flat, trainer, ln, idr, tm, gF, gV):
        B, N, S = ln.shape
        dev = idr.device
        A = torch.empty(B * N, 4 * _dp.E, dtype=idr.dtype, device=dev)
        Ad = torch.empty_like(A)
        flat = emb_flat.detach().contiguous()
        m = trainer._struct(flat)
        _check(_lib.load().matpl_dp_dual_forward(
            trainer.code, ctypes.byref(m), B, N, S, _ptr(ln), _ptr(idr), _ptr(tm), _ptr(gF),
            _ptr(gV), _ptr(A), _ptr(Ad), torch.cuda.current_stream(dev).cuda_stream),
            "matpl_dp_dual_forward")
        ctx.trainer = trainer
        ctx.save_for_backward(flat, ln, idr, tm, gF, gV if gV is not None else flat[:0])
        ctx.has_gv = gV is not None
        return A, Ad

    @staticmethod
    @_lib.on_device
    def backward(ctx, gA, gAd):
        flat, ln, idr, tm, gF, gV = ctx.saved_tensors
        B, N, S = ln.shape
        dev = idr.device
        gA = torch.zeros_like(flat[:0].new_empty(B * N, 4 * _dp.E)) if gA is None else gA.contiguous()
        gAd = torch.zeros_like(gA) if gAd is None else gAd.contiguous()
        grad = torch.empty_like(flat)
        m = ctx.trainer._struct(flat)
        _check(_lib.load().matpl_dp_dual_backward(
            ctx.trainer.code, ctypes.byref(m), B, N, S, _ptr(ln), _ptr(idr), _ptr(tm), _ptr(gF),
            _ptr(gV) if ctx.has_gv else 0, _ptr(gA), _ptr(gAd), _ptr(grad),
            torch.cuda.current_stream(dev).cuda_stream), "matpl_dp_dual_backward")
        return grad, None, None, None, None, None, None


class _EmptySlots(torch.autograd.Function):
    """A = A_occ + the empty-slot term of A (matpl_dp_pad_forward: every empty slot of type
    block t_j holds the normalised zero row, whose embedding is the same for all of them); the
    backward passes dPhi/dA to A_occ unchanged and gives the embedding parameters' part through
    the empty slots (matpl_dp_pad_backward)."""

    @staticmethod
    @_lib.on_device
    def forward(ctx, A_occ, emb_flat, trainer, ln, tm):
        B, N, S = ln.shape
        dev = ln.device
        A_occ = A_occ.contiguous()
        flat = emb_flat.detach().contiguous()
        m = trainer._struct(flat)
        L = _lib.load()
        np_ = len(trainer._present)
        ws = torch.empty(L.matpl_dp_pad_workspace_bytes(np_), dtype=torch.uint8, device=dev)
        ne = torch.empty(B * N, np_, dtype=torch.int32, device=dev)
        A = torch.empty_like(A_occ)
        _check(L.matpl_dp_pad_forward(
            trainer.code, ctypes.byref(m), B, N, S, _ptr(ln), _ptr(tm), _ptr(A_occ), _ptr(A),
            _ptr(ne), _ptr(ws), ws.numel(), torch.cuda.current_stream(dev).cuda_stream),
            "matpl_dp_pad_forward")
        ctx.trainer, ctx.shape = trainer, (B, N, S)
        ctx.save_for_backward(flat, tm, ne, ws)
        return A

    @staticmethod
    @_lib.on_device
    def backward(ctx, gA):
        flat, tm, ne, ws = ctx.saved_tensors
        B, N, S = ctx.shape
        gA = gA.contiguous()
        grad = torch.empty_like(flat)
        m = ctx.trainer._struct(flat)
        _check(_lib.load().matpl_dp_pad_backward(
            ctx.trainer.code, ctypes.byref(m), B, N, S, _ptr(tm), _ptr(ne), _ptr(gA),
            _ptr(grad), _ptr(ws), ws.numel(), torch.cuda.current_stream(gA.device).cuda_stream),
            "matpl_dp_pad_backward")
        return gA, grad, None, None, None


class _DescDual(torch.autograd.Function):
    """(D, D_dot) = (A^T A<, A_dot^T A< + A^T A_dot<) for the atoms rows (matpl_dp_desc_dual,
    output row r = atom rows[r]); the backward is the transpose map (matpl_dp_desc_dual_grad)."""

    @staticmethod
    @_lib.on_device
    def forward(ctx, A, Ad, m2, rows):
        A = A.contiguous()
        Ad = Ad.contiguous()
        R = rows.numel()
        D = torch.empty(R, _dp.E, m2, dtype=A.dtype, device=A.device)
        Dd = torch.empty_like(D)
        code = _lib.MATPL_F64 if A.dtype == torch.float64 else _lib.MATPL_F32
        _check(_lib.load().matpl_dp_desc_dual(code, R, m2, _ptr(rows), _ptr(A), _ptr(Ad), _ptr(D),
                                              _ptr(Dd),
                                              torch.cuda.current_stream(A.device).cuda_stream),
               "matpl_dp_desc_dual")
        ctx.save_for_backward(A, Ad, rows)
        ctx.m2 = m2
        return D, Dd

    @staticmethod
    @torch.autograd.function.once_differentiable
    @_lib.on_device
    def backward(ctx, gD, gDd):
        A, Ad, rows = ctx.saved_tensors
        R = rows.numel()
        full = R == A.shape[0]               # a permutation of every atom writes every row
        gA = torch.empty_like(A) if full else torch.zeros_like(A)
        gAd = torch.empty_like(Ad) if full else torch.zeros_like(Ad)
        code = _lib.MATPL_F64 if A.dtype == torch.float64 else _lib.MATPL_F32
        gD = gD.contiguous() if gD is not None else None
        gDd = gDd.contiguous() if gDd is not None else None
        _check(_lib.load().matpl_dp_desc_dual_grad(
            code, R, ctx.m2, _ptr(rows), _ptr(A), _ptr(Ad), _ptr(gD), _ptr(gDd), _ptr(gA),
            _ptr(gAd), torch.cuda.current_stream(A.device).cuda_stream), "matpl_dp_desc_dual_grad")
        return gA, gAd, None, None


# fitting parameters in the order of the packed fitting block (dp_layout.cuh FitOff) with their
# (offset, size) there
_FIT_PARAMS = (("0.weight", _dp.FIT_W0, _dp.DIN * _dp.F), ("0.bias", _dp.FIT_B0, _dp.F),
               ("1.weight", _dp.FIT_W1, _dp.F * _dp.F), ("1.bias", _dp.FIT_B1, _dp.F),
               ("1.resnet_dt", _dp.FIT_DT1, _dp.F), ("2.weight", _dp.FIT_W2, _dp.F * _dp.F),
               ("2.bias", _dp.FIT_B2, _dp.F), ("2.resnet_dt", _dp.FIT_DT2, _dp.F),
               ("3.weight", _dp.FIT_W3, _dp.F), ("3.bias", _dp.FIT_B3, 1))


class _FitDualPhi(torch.autograd.Function):
    """phi = sum_r (a_r E_r + E_dot_r) over the element blocks of the rows (D, D_dot) (each
    element's fitting net, dp_embedding.py:140-163, on both streams) together with its
    first-order gradient in D, D_dot and the fitting parameters, all from matpl_dp_fit_dual, one
    launch pair per element into one gradient buffer (the blocks are disjoint row ranges, so no
    zero fill, no accumulation).  ``blocks`` = ((row offset, rows, element), ...); ``packed`` =
    the evaluator's packed parameters (current weights, with the transposed matrices) of which
    element t's fitting block starts at woff + t FIT_SIZE; ``params`` = the fitting parameter
    tensors of every block's element, ``len(_FIT_PARAMS)`` per block.  The backward scales the
    stored gradients by the incoming one."""

    @staticmethod
    @_lib.on_device
    def forward(ctx, D, Dd, a, packed, blocks, woff, *params):
        from .ops import workspace
        dev = D.device
        D, Dd, a = D.contiguous(), Dd.contiguous(), a.contiguous()
        gD = torch.empty_like(D)
        gDd = torch.empty_like(Dd)
        npar = _dp.FIT_B3 + 1
        gP = torch.zeros(len(blocks), npar, dtype=D.dtype, device=dev)
        phi = torch.zeros(1, dtype=torch.float64, device=dev)
        code = _lib.MATPL_F64 if D.dtype == torch.float64 else _lib.MATPL_F32
        lib = _lib.load()
        stream = torch.cuda.current_stream(dev).cuda_stream
        nmax = max(n for _, n, _ in blocks)
        ws = workspace(dev, lib.matpl_dp_fit_dual_workspace_bytes(code, nmax), "fit_dual")
        es = D.element_size()
        for b, (o, n, t) in enumerate(blocks):
            blk = packed[woff + t * _dp.FIT_SIZE:woff + (t + 1) * _dp.FIT_SIZE]
            row = o * D.shape[1] * es
            _check(lib.matpl_dp_fit_dual(code, n, _ptr(blk), _ptr(D) + row, _ptr(Dd) + row,
                                         _ptr(a) + o * es, _ptr(gD) + row, _ptr(gDd) + row,
                                         _ptr(gP[b]), _ptr(phi), _ptr(ws), ws.numel(), stream),
                   "matpl_dp_fit_dual")
        ctx.save_for_backward(gD, gDd, gP)
        ctx.shapes = [p.shape if p is not None else None for p in params]
        return phi.to(D.dtype).reshape(())

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, gphi):
        gD, gDd, gP = ctx.saved_tensors
        torch._foreach_mul_([gD, gDd, gP], gphi)        # one launch for the three buffers
        grads = []
        k = len(_FIT_PARAMS)
        for q, shape in enumerate(ctx.shapes):
            _, off, size = _FIT_PARAMS[q % k]
            grads.append(None if shape is None else gP[q // k, off:off + size].reshape(shape))
        return (gD, gDd, None, None, None, None, *grads)


class FusedTrainer:
    """Force-loss training step with the embedding nets' second-order gradient in this
    library's kernels.  Per composition cluster (as ``dp_trainer.train``):

    1. E, F with the current parameters through the fused evaluation (``matpl_dp_eval``);
    2. gE = dL/dE, gF = dL/dF of the loss (dp_loss's MSE terms) on those values;
    3. A, A_dot = per-atom descriptor factor and its tangent along the seed gF
       (``matpl_dp_dual_forward``), plus the empty-slot term of A
       (``matpl_dp_pad_forward``);
    4. Ei = fitting nets on D = A^T A<, Edot = dEi/dA . A_dot;
    5. Phi = sum gE Etot + sum Edot; Phi.backward() gives dL/dtheta: the fitting part by
       ``matpl_dp_fit_dual`` (both streams and the closed-form reverse pass in one kernel, the
       weight gradients as row sums in a second), the embedding part by
       ``matpl_dp_dual_backward``.

    ``model`` is a DPTrainModel (its Parameters are trained), float32 or float64.
    ``eval_precision``: the form of step 1's evaluation, which only seeds gE and gF; None = the
    model's dtype; "mixed" (float32 models) runs it on the tcgen05 tensor cores (BF16x3
    operands, FP32 accumulation; E / F within ~1e-5 relative of FP32, so the gradient moves by
    that much relative to the loss residuals).
    ``fit_kernel``: False runs steps 4-5 of the fitting part as torch operations and autograd
    (the same mathematics; kept for comparison and for fitting shapes other than the compiled
    400-50-50-50-1)."""

    def __init__(self, model: DPTrainModel, eval_precision: Optional[str] = None,
                 fit_kernel: bool = True):
        if model.dtype not in (torch.float32, torch.float64):
            raise _lib.MatplError("FusedTrainer needs a float32 or float64 DPTrainModel")
        self.model = model
        cfg = model.cfg
        self.code = _lib.MATPL_F64 if model.dtype == torch.float64 else _lib.MATPL_F32
        prec = "float64" if model.dtype == torch.float64 else "float32"
        if eval_precision is not None and eval_precision != prec:
            if model.dtype != torch.float32 or not eval_precision.startswith("mixed"):
                raise _lib.MatplError("eval_precision: a mixed form for a float32 model, or the "
                                      "model's own dtype")
            prec = eval_precision
        self.eval_precision = prec
        dev = model.davg.device
        self.evaluator = _dp.DP(cfg, {}, model.davg.cpu(), model.dstd.cpu(), precision=prec,
                                device=dev, check_errors=False, packed=_pack_device(model))
        self.davg4 = self.evaluator.davg4
        self.dstd4 = self.evaluator.dstd4
        self._present = None
        compiled = (list(cfg.fit_sizes) == [_dp.F] * 3 + [1] and cfg.M2 == _dp.M2 and
                    list(cfg.emb_sizes) == [_dp.E] * 3)
        self.fit_kernel = bool(fit_kernel) and compiled

    def _struct(self, flat):
        m = _lib.MatplDpModel()
        cfg = self.model.cfg
        m.ntypes, m.m = cfg.ntypes, cfg.maxNeighborNum
        m.npresent = len(self._present)
        for q, t in enumerate(self._present):
            m.present[q] = t
        m.rmin, m.rmax = float(cfg.Rmin), float(cfg.Rmax)
        m.params, m.davg, m.dstd = _ptr(flat), _ptr(self.davg4), _ptr(self.dstd4)
        m.err_dev = _ptr(self.evaluator.err)
        return m

    def _fit_dual(self, t: int, x: torch.Tensor, xd: torch.Tensor):
        """Fitting net of element t (dp_embedding.py:140-163) on rows x and its tangent xd:
        (E, Edot) per row.  Primal and tangent share each matrix product."""
        model, cfg = self.model, self.model.cfg
        nl = len(cfg.fit_sizes)
        n = x.shape[0]
        for l in range(nl - 1):
            pre = f"fitting_net.{t}.layers.{l}."
            zz = splitk.mm(torch.cat([x, xd], 0), model.param(pre + "weight"))
            z, zd = zz[:n], zz[n:]
            b = model.param(pre + "bias")
            if b is not None:
                z = splitk.add_row(z, b)
            h = torch.tanh(z)
            hd = (1 - h * h) * zd
            if l == 0:
                x, xd = h, hd
            else:
                dt = model.param(pre + "resnet_dt")
                if dt is not None:
                    h, hd = h * dt, hd * dt
                x, xd = h + x, hd + xd
        pre = f"fitting_net.{t}.layers.{nl - 1}."
        ee = splitk.mm(torch.cat([x, xd], 0), model.param(pre + "weight"))
        e, ed = ee[:n], ee[n:]
        b = model.param(pre + "bias")
        return (splitk.add_row(e, b) if b is not None else e), ed

    def _type_index(self, tm32: torch.Tensor, present, B: int):
        """Atom rows of the [B*N] batch grouped by present element, b-major inside each
        element ([B, n] blocks), and each element's (start, count) in that order (cached per
        type map and batch size: one host sync when it changes)."""
        key = (self._tm_src.data_ptr(), tm32.numel(), tuple(present), B)
        if getattr(self, "_tidx_key", None) != key:
            tl = tm32.long()
            N = tl.numel()
            base = torch.arange(B, device=tl.device).reshape(B, 1) * N
            rows, blocks, off = [], {}, 0
            for ti in present:
                idx = torch.nonzero(tl == ti).flatten()
                n = idx.numel()
                rows.append((base + idx.reshape(1, n)).reshape(-1))
                blocks[ti] = (off, n)
                off += B * n
            self._rows = torch.cat(rows).contiguous()
            self._blocks = blocks
            self._tidx_key = key
        return self._rows, self._blocks

    def _loss_and_backward(self, batch: dict, w_f: float, w_e: float):
        """Steps 1-5 with device tensors only (no host synchronisation once the type index is
        cached): returns (loss, le, lf) as 0-d tensors and leaves the gradients in .grad."""
        model, cfg = self.model, self.model.cfg
        ln = batch["list_neigh"]
        B, N, S = ln.shape
        dev = ln.device
        ln32 = ln if ln.dtype == torch.int32 and ln.is_contiguous() else ln.to(torch.int32).contiguous()
        idr = batch["ImageDR"]
        idr = idr if idr.dtype == model.dtype and idr.is_contiguous() else idr.to(model.dtype).contiguous()
        tm32 = batch["type_map"]
        self._tm_src = tm32
        tm32 = tm32 if tm32.dtype == torch.int32 else tm32.to(device=dev, dtype=torch.int32).contiguous()
        present = [cfg.atom_type.index(int(a)) for a in batch["atom_type"]
                   if int(a) in cfg.atom_type]
        self._present = present
        rows, blocks = self._type_index(tm32, present, B)
        # 1. E, F with the current parameters
        self.evaluator.packed.copy_(_pack_device(model))
        r = self.evaluator.evaluate(ln32, tm32, present, idr, 0)
        # 2. loss gradient w.r.t. E and F (a ragged batch: E per configuration)
        ragged = "config_of_atom" in batch
        if ragged:
            from .data import config_energies
            cfg_of = batch["config_of_atom"]
            C = batch["Etot"].numel()
            Et = config_energies(r["Ei_atom"].to(model.dtype), cfg_of, C).detach().requires_grad_()
            E_lab = batch["Etot"].to(model.dtype).reshape(C)
        else:
            Et = r["Etot"].to(model.dtype).reshape(B, 1).detach().requires_grad_()
            E_lab = batch["Etot"].to(model.dtype).reshape(B, 1)
        Fo = r["Force"].detach().requires_grad_()
        le = torch.nn.functional.mse_loss(Et, E_lab)
        lf = torch.nn.functional.mse_loss(Fo, batch["Force"].to(model.dtype))
        loss = w_e * le + w_f * lf
        gE, gF = torch.autograd.grad(loss, [Et, Fo])
        gF = gF.contiguous()
        # 3. descriptor factor and its tangent
        emb = _emb_flat(model)
        A_occ, Ad = _EmbedDual.apply(emb, self, ln32, idr, tm32, gF, None)
        A = _EmptySlots.apply(A_occ, emb, self, ln32, tm32).reshape(B, N, 4, _dp.E)
        Ad = Ad.reshape(B, N, 4, _dp.E)
        # 4. per-atom energies and their tangent (explicit forward-mode through D and the
        #    fitting net), 5. one first-order backward of Phi gives every parameter gradient
        # D rows grouped by element (b-major inside each element): every fitting net reads a
        # contiguous block, no gather / scatter
        D_all, Dd_all = _DescDual.apply(A.reshape(B * N, 4, _dp.E), Ad.reshape(B * N, 4, _dp.E),
                                        cfg.M2, rows)
        D_all = D_all.reshape(D_all.shape[0], -1)
        Dd_all = Dd_all.reshape(Dd_all.shape[0], -1)
        phi = A.new_zeros(())
        if self.fit_kernel:
            # every element block in one autograd node (disjoint row ranges of D_all)
            if ragged:          # dL/dE of each row's configuration
                a_all = gE.index_select(0, cfg_of.index_select(0, rows.remainder(N)))
            else:               # rows are b * N + i
                a_all = gE.reshape(B).index_select(0, torch.div(rows, N, rounding_mode="floor"))
            fb, params = [], []
            for ti in present:
                o, n = blocks[ti]
                if n == 0:
                    continue
                fb.append((o, B * n, ti))
                params += [model.param(f"fitting_net.{ti}.layers.{nm}") for nm, _, _ in _FIT_PARAMS]
            woff = cfg.ntypes * cfg.ntypes * _dp.EMB_SIZE
            phi = _FitDualPhi.apply(D_all, Dd_all, a_all.to(model.dtype).detach(),
                                    self.evaluator.packed, tuple(fb), woff, *params)
        for ti in present if not self.fit_kernel else ():
            o, n = blocks[ti]
            if n == 0:
                continue
            e, ed = self._fit_dual(ti, D_all[o:o + B * n], Dd_all[o:o + B * n])
            if ragged:          # dL/dE of each row's configuration
                gr = gE.index_select(0, cfg_of.index_select(0, rows[o:o + n]))
                phi = phi + (gr * e.reshape(-1)).sum() + ed.sum()
            else:
                phi = phi + (gE.reshape(B, 1) * e.reshape(B, n)).sum() + ed.sum()
        phi.backward()
        return loss.detach(), le.detach(), lf.detach()

    def loss_and_backward(self, batch: dict, w_f: float = 1.0, w_e: float = 1.0):
        loss, le, lf = self._loss_and_backward(batch, w_f, w_e)
        return float(loss), float(le), float(lf)

    def step(self, batches, optimizer, w_f: float = 1.0, w_e: float = 1.0):
        total = 0.0
        for b in batches:
            optimizer.zero_grad(set_to_none=True)
            l, _, _ = self.loss_and_backward(b, w_f, w_e)
            optimizer.step()
            total += l
        return total


class GraphedTrainer:
    """The fused training step (FusedTrainer) captured once per batch shape in a CUDA graph:
    loss, both dual kernels, the fitting part, the backward and the optimizer update replay as
    one graph launch, so the step costs no host work beyond copying the batch into the graph's
    static buffers.  The optimizer must keep its state on the device (torch.optim.Adam /
    AdamW with capturable=True, or SGD).  ``step`` returns the loss as a device tensor."""

    KEYS = ("list_neigh", "ImageDR", "type_map", "Etot", "Force")

    def __init__(self, trainer: FusedTrainer, optimizer: torch.optim.Optimizer,
                 w_f: float = 1.0, w_e: float = 1.0, warmup: int = 3):
        self.tr, self.opt = trainer, optimizer
        self.w_f, self.w_e, self.warmup = w_f, w_e, warmup
        self.graphs = {}

    def _keys(self, batch):
        return self.KEYS + (("config_of_atom",) if "config_of_atom" in batch else ())

    def _capture(self, batch):
        static = {k: batch[k].clone() for k in self._keys(batch)}
        static["atom_type"] = list(batch["atom_type"])
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(self.warmup):            # allocator, workspaces, type index, attrs
                self.opt.zero_grad(set_to_none=True)
                self.tr._loss_and_backward(static, self.w_f, self.w_e)
                self.opt.step()
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        self.opt.zero_grad(set_to_none=True)
        with torch.cuda.graph(g, stream=side):   # the warm-up's workspaces are reused
            loss, le, lf = self.tr._loss_and_backward(static, self.w_f, self.w_e)
            self.opt.step()
        return g, static, loss

    def step(self, batch):
        keys = self._keys(batch)
        key = tuple(tuple(batch[k].shape) for k in keys) + (tuple(batch["atom_type"]),)
        if key not in self.graphs:
            self.graphs[key] = self._capture(batch)
        g, static, loss = self.graphs[key]
        for k in keys:
            if batch[k].data_ptr() != static[k].data_ptr():
                static[k].copy_(batch[k], non_blocking=True)
        g.replay()
        return loss
