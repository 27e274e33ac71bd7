"""ORACLE — test infrastructure only (see ``oracle/__init__.py``).

torch-FP64 (or FP32) CPU restatement of MatPL's DP se_e2_a evaluation, the path of
``src/model/dp_dp_script.py`` (identical math to ``src/model/dp_dp.py`` on CPU):

* environment matrix         ``dp_dp.py:217-302``   (``calculate_Ri``)
* embedding nets             ``dp_embedding.py:73-94``
* descriptor contraction     ``dp_dp.py:344-415``   (``calculate_xyz_scater``)
* fitting nets               ``dp_embedding.py:140-163`` and ``dp_dp.py:304-342``
* dE/dRi by autograd and the CPU force/virial scatter  ``dp_dp.py:417-459``

Weights are passed as a mapping with the reference's own ``state_dict`` key names
(``embedding_net.{k}.layers.{l}.weight`` ...), so a reference checkpoint or TorchScript
``jit_dp.pt`` state dict can be used directly.  Autograd builds the same derivative graph
the reference builds; the oracle is pinned against outputs of the reference itself
(``tests/golden``).
"""
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import torch


@dataclass
class DPConfig:
    """Hyper-parameters the reference reads from its JSON config (``dp_dp.py:44-85``)."""
    atom_type: List[int]                 # model element list, e.g. [29] or [3, 14]
    Rmax: float = 6.0                    # config["Rc_M"]
    Rmin: float = 0.5                    # config["atomType"][0]["Rm"]
    maxNeighborNum: int = 100            # m, slots per neighbor type
    M2: int = 16
    emb_sizes: List[int] = field(default_factory=lambda: [25, 25, 25])
    fit_sizes: List[int] = field(default_factory=lambda: [50, 50, 50, 1])

    @property
    def ntypes(self) -> int:
        return len(self.atom_type)


def _present_types(cfg: DPConfig, atom_type) -> List[int]:
    """Model type index of each image type (``dp_dp.py:145-165``)."""
    out = []
    for a in [int(x) for x in atom_type]:
        if a in cfg.atom_type:
            out.append(cfg.atom_type.index(a))
    return out


def env_matrix(cfg: DPConfig, ImageDR: torch.Tensor, Imagetype_map: torch.Tensor,
               davg: torch.Tensor, dstd: torch.Tensor):
    """Normalised Ri [B,N,S,4] and Ri_d [B,N,S,4,3] (``dp_dp.py:217-302``)."""
    R = ImageDR[..., 0]
    x, y, z = ImageDR[..., 1], ImageDR[..., 2], ImageDR[..., 3]
    rmin, rmax = cfg.Rmin, cfg.Rmax
    inner = (R > 0) & (R < rmin)
    shell = (R > rmin) & (R < rmax)
    Rsafe = torch.where(R != 0, R, torch.ones_like(R))
    u = (Rsafe - rmin) / (rmax - rmin)
    poly = u ** 3 * (-6 * u ** 2 + 15 * u - 10) + 1
    dpoly = (3 * u ** 2 * (-6 * u ** 2 + 15 * u - 10) + u ** 3 * (-12 * u + 15)) / (rmax - rmin)
    s = torch.where(inner, 1 / Rsafe, torch.where(shell, poly / Rsafe, torch.zeros_like(R)))
    ds = torch.where(inner, -1 / Rsafe ** 2,
                     torch.where(shell, dpoly / Rsafe - poly / Rsafe ** 2, torch.zeros_like(R)))
    mask = R.abs() > 1e-5
    zero = torch.zeros_like(R)
    Ri = torch.stack([s,
                      torch.where(mask, s * x / Rsafe, zero),
                      torch.where(mask, s * y / Rsafe, zero),
                      torch.where(mask, s * z / Rsafe, zero)], dim=-1)
    common = (ds - s / Rsafe) / Rsafe ** 2
    xyz = [x, y, z]
    cols = []
    for b in range(3):          # derivative w.r.t. x, y, z of the pair vector
        rb = xyz[b]
        col = [torch.where(mask, ds * rb / Rsafe, zero)]
        for a in range(3):
            v = common * xyz[a] * rb
            if a == b:
                v = v + s / Rsafe
            col.append(torch.where(mask, v, zero))
        cols.append(torch.stack(col, dim=-1))       # [B,N,S,4]
    dfeat = torch.stack(cols, dim=-1)                # [B,N,S,4,3]
    B, N, S = R.shape
    davg_a = davg.to(R.dtype)[Imagetype_map.long()].reshape(N, S, 4)
    dstd_a = dstd.to(R.dtype)[Imagetype_map.long()].reshape(N, S, 4)
    Ri = (Ri - davg_a) / dstd_a
    Ri_d = -dfeat / dstd_a.unsqueeze(-1)
    return Ri, Ri_d


def _emb_forward(params: Dict[str, torch.Tensor], k: int, sizes: List[int], s: torch.Tensor):
    """Embedding net ``k`` on s [..., 1] (``dp_embedding.py:73-94``)."""
    widths = [1] + list(sizes)
    x = s
    for l in range(len(sizes)):
        pre = f"embedding_net.{k}.layers.{l}."
        h = x @ params[pre + "weight"]
        if pre + "bias" in params:
            h = h + params[pre + "bias"]
        h = torch.tanh(h)
        dt = params.get(pre + "resnet_dt")
        if widths[l + 1] == widths[l]:
            x = (h * dt if dt is not None else h) + x
        elif widths[l + 1] == 2 * widths[l]:
            x = torch.cat((x, x), dim=-1) + (h * dt if dt is not None else h)
        else:
            x = h
    return x


def _fit_forward(params: Dict[str, torch.Tensor], t: int, sizes: List[int], x: torch.Tensor):
    """Fitting net ``t`` (``dp_embedding.py:140-163``)."""
    nl = len(sizes)
    for l in range(nl - 1):
        pre = f"fitting_net.{t}.layers.{l}."
        h = x @ params[pre + "weight"]
        if pre + "bias" in params:
            h = h + params[pre + "bias"]
        h = torch.tanh(h)
        if l == 0:
            x = h
        else:
            dt = params.get(pre + "resnet_dt")
            x = (h * dt if dt is not None else h) + x
    pre = f"fitting_net.{t}.layers.{nl - 1}."
    y = x @ params[pre + "weight"]
    if pre + "bias" in params:
        y = y + params[pre + "bias"]
    return y


def energy_from_Ri(cfg: DPConfig, params, Ri: torch.Tensor, Imagetype_map: torch.Tensor,
                   present: List[int]):
    """Ei in the reference's type-grouped order, plus Ei in atom order (zeros for atoms whose
    type is absent).  ``dp_dp.py:304-415``."""
    B, N, S, _ = Ri.shape
    m = cfg.maxNeighborNum
    T = len(present)
    tmap = Imagetype_map.long().flatten()
    Ei_blocks = []
    Ei_atom = torch.zeros(B, N, 1, dtype=Ri.dtype)
    for ti in present:
        idx = torch.nonzero(tmap == ti).flatten()
        if idx.numel() == 0:
            continue
        A = None
        for tj in present:
            blk = Ri[:, idx, tj * m:(tj + 1) * m, :]             # [B, n, m, 4]
            G = _emb_forward(params, ti * cfg.ntypes + tj, cfg.emb_sizes, blk[..., 0:1])
            c = blk.transpose(-2, -1) @ G                          # [B, n, 4, E]
            A = c if A is None else A + c
        A = A / (m * T)
        D = A.transpose(-2, -1) @ A[..., :cfg.M2]                  # [B, n, E, M2]
        Ei_t = _fit_forward(params, ti, cfg.fit_sizes, D.reshape(B, idx.numel(), -1))
        Ei_blocks.append(Ei_t)
        Ei_atom = Ei_atom.index_copy(1, idx, Ei_t)
    return torch.cat(Ei_blocks, dim=1), Ei_atom


def dp_eval(cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
            list_neigh, Imagetype_map, atom_type, ImageDR, nghost: int = 0,
            virial_convention: str = "cpu", create_graph: bool = False):
    """Energy, forces and virial exactly as ``DP.forward`` on CPU returns them.

    list_neigh [B,N,S] int (1-based, 0 = empty); ImageDR [B,N,S,4]; returns a dict with
    Etot [B,1], Ei [B,N] (type-grouped order), Ei_atom [B,N], Force [B,N+nghost,3],
    Virial [B,9], dE [B,N,S,4] (dE/dRi of the normalised Ri).
    ``virial_convention``: "cpu" = upper triangle Rij_a*f_b mirrored (``dp_dp.py:448-458``);
    "gpu" = all nine f_a*Rij_b (``src/op/kernel/calculateVirial.cu:80``).
    """
    dtype = ImageDR.dtype
    ImageDR = ImageDR.detach()
    B, N, S, _ = ImageDR.shape
    present = _present_types(cfg, atom_type)
    Ri, Ri_d = env_matrix(cfg, ImageDR, Imagetype_map, davg, dstd)
    Ri = Ri.detach().requires_grad_()
    Ei, Ei_atom = energy_from_Ri(cfg, params, Ri, Imagetype_map, present)
    Etot = Ei.sum(1)
    dE = torch.autograd.grad([Etot], [Ri], grad_outputs=[torch.ones_like(Etot)],
                             create_graph=create_graph, retain_graph=create_graph)[0]
    dE_Rid = (dE.unsqueeze(-1) * Ri_d).sum(-2)                   # [B,N,S,3]
    Force = torch.zeros(B, N + nghost + 1, 3, dtype=dtype)
    Force[:, 1:N + 1] = -dE_Rid.sum(-2)
    for b in range(B):
        idx = list_neigh[b].reshape(-1, 1).long().expand(-1, 3)
        Force[b] = Force[b].scatter_add(0, idx, dE_Rid[b].reshape(-1, 3))
    Force = Force[:, 1:]
    Rij = ImageDR[..., 1:]
    if virial_convention == "cpu":
        V = torch.zeros(B, 9, dtype=dtype)
        for a in range(3):
            for c in range(a, 3):
                V[:, 3 * a + c] = (Rij[..., a] * dE_Rid[..., c]).reshape(B, -1).sum(1)
        V[:, 3], V[:, 6], V[:, 7] = V[:, 1], V[:, 2], V[:, 5]
    else:
        V = torch.einsum("bnsa,bnsc->bac", dE_Rid, Rij).reshape(B, 9)
    return {"Etot": Etot, "Ei": Ei.squeeze(-1), "Ei_atom": Ei_atom.squeeze(-1), "Force": Force,
            "Virial": V, "dE": dE, "Ri": Ri, "Ri_d": Ri_d}


def dp_eval_chunked(cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
                    list_neigh, Imagetype_map, atom_type, ImageDR, chunk: int = 2000):
    """``dp_eval`` for one large image, in chunks of centre atoms (the same arithmetic: the
    energy is a sum of per-atom terms, each depending on its own row of Ri only, and every
    row's dE/dRi contracts with Ri_d into the centre and neighbor forces,
    ``dp_dp.py:417-459``).  Bounds the autograd graph to ``chunk`` centre atoms.  Returns
    Etot [1], Ei_atom [1,N], Force [1,N,3] and Virial [1,9] (all nine f_a*Rij_b, the GPU
    operator's convention, ``calculateVirial.cu:80``)."""
    dtype = ImageDR.dtype
    B, N, S, _ = ImageDR.shape
    assert B == 1
    present = _present_types(cfg, atom_type)
    tmap = Imagetype_map.reshape(-1)
    Force = torch.zeros(N + 1, 3, dtype=dtype)
    V = torch.zeros(3, 3, dtype=dtype)
    Ei_atom = torch.zeros(N, dtype=dtype)
    for c0 in range(0, N, chunk):
        c1 = min(N, c0 + chunk)
        idr = ImageDR[:, c0:c1].detach()
        Ri, Ri_d = env_matrix(cfg, idr, tmap[c0:c1], davg, dstd)
        Ri = Ri.detach().requires_grad_()
        _, ea = energy_from_Ri(cfg, params, Ri, tmap[c0:c1], present)
        e = ea.sum()
        dE = torch.autograd.grad([e], [Ri])[0]
        f = (dE.unsqueeze(-1) * Ri_d).sum(-2)[0]                  # [n, S, 3]
        Ei_atom[c0:c1] = ea.detach().reshape(-1)
        Force[1 + c0:1 + c1] -= f.sum(-2)
        Force.index_add_(0, list_neigh[0, c0:c1].reshape(-1).long(), f.reshape(-1, 3))
        V += torch.einsum("nsa,nsc->ac", f, idr[0, ..., 1:])
    return {"Etot": Ei_atom.sum().reshape(1), "Ei_atom": Ei_atom.reshape(1, N),
            "Force": Force[1:].reshape(1, N, 3), "Virial": V.reshape(1, 9)}


def force_virial_ops(list_neigh0, dE, Ri_d, Rij, F_center, nghost: int):
    """Oracle for the ``calculateForce`` / ``calculateVirial`` custom ops
    (``src/op/src/CalcOps.cpp:6-22, 170-185``; kernels ``calculateForce.cu:49-93``,
    ``calculateVirial.cu:19-86``).

    list_neigh0 [B,N,S] int, 0-based, -1 = empty; dE [B,N,4S]; Ri_d [B,N,4S,3]; Rij [B,N,S,3];
    F_center [B,N,3].  Returns (force [B,N+nghost,3], virial [B,9], atom_virial [B,N+nghost,9]).
    The reference's force kernel strides the batch by N, not N+nghost
    (``calculateForce.cu:90``); for B == 1 or nghost == 0 the two agree, and this oracle uses
    the N+nghost stride, which is the layout of the tensor the op returns.
    """
    B, N, S = list_neigh0.shape
    dE4 = dE.reshape(B, N, S, 4)
    Rd = Ri_d.reshape(B, N, S, 4, 3)
    f = (dE4.unsqueeze(-1) * Rd).sum(-2)                      # [B,N,S,3]
    force = torch.zeros(B, N + nghost, 3, dtype=dE.dtype)
    force[:, :N] = F_center
    av = torch.zeros(B, N + nghost, 9, dtype=dE.dtype)
    pv = torch.einsum("bnsa,bnsc->bnsac", f, Rij).reshape(B, N, S, 9)
    for b in range(B):
        nl = list_neigh0[b].reshape(-1).long()
        ok = nl >= 0
        force[b].index_add_(0, nl[ok], f[b].reshape(-1, 3)[ok])
        av[b].index_add_(0, nl[ok], pv[b].reshape(-1, 9)[ok])
    return force, av.sum(1), av


def force_virial_grads(list_neigh0, Ri_d, Rij, grad_force, grad_virial):
    """Oracle for ``CalculateForce::backward`` and ``CalculateVirial::backward``
    (``src/op/kernel/calculateForceGrad.cu:10-90``, ``calculateVirialGrad.cu:16-92``).
    Returns (grad_dE_from_force, grad_dE_from_virial), each [B,N,4S]."""
    B, N, S = list_neigh0.shape
    Rd = Ri_d.reshape(B, N, S, 4, 3)
    gF = grad_force[:, :N]                                     # [B,N,3]
    gf_center = -(Rd * gF[:, :, None, None, :]).sum(-1)        # [B,N,S,4]
    nl = list_neigh0.long()
    ok = nl >= 0
    jj = torch.where(ok, nl % N, torch.zeros_like(nl))
    gj = torch.stack([gF[b][jj[b]] for b in range(B)])         # [B,N,S,3]
    gf_nei = (Rd * gj[:, :, :, None, :]).sum(-1) * ok[..., None]
    gV = grad_virial.reshape(B, 3, 3)
    gvir = torch.einsum("bac,bnsc,bnswa->bnsw", gV, Rij, Rd) * ok[..., None]
    return (gf_center + gf_nei).reshape(B, N, 4 * S), gvir.reshape(B, N, 4 * S)


def compress_oracle(f2, coefficient):
    """Oracle for ``calculateCompress`` and its backward (``src/op/kernel/calculateCompress.cu:3-55``,
    ``calculateCompress_grad.cu:3-53``, ``CalcOps.cpp:343-356``): G = sum_k c_k f2^(n-1-k), and
    dG/df2, evaluated term by term in float64."""
    f = f2.reshape(-1, 1).to(torch.float64)
    c = coefficient.to(torch.float64)
    n = c.shape[-1]
    G = torch.zeros(c.shape[:2], dtype=torch.float64)
    dG = torch.zeros(c.shape[:2], dtype=torch.float64)
    for k in range(n):
        p = n - 1 - k
        G = G + c[..., k] * f ** p
        if p > 0:
            dG = dG + p * c[..., k] * f ** (p - 1)
    return G, dG
