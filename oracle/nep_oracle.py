"""ORACLE - test infrastructure only (see ``oracle/__init__.py``): never imported by the product.

FP64 CPU restatement of MatPL's NEP evaluation path.

* ``neighbor`` / ``maxneigh``: ctypes glue around ``nepneigh.c`` (the restatement of
  ``CalcOps_cpu.calculate_neighbor`` / ``calculate_maxneigh``, src/op/src/CalcOps_cpu.cpp:100-185).
* ``features``: the descriptor of ``NEP.calculate_qn`` (src/model/nep_net.py:648-838):
  Chebyshev radial functions ``cal_fk`` (:691-715), two-body q_n = sum_j sum_k c2 f_k
  (``cal_feat_2body`` :717-730), angular s_nlm = sum_j g_n(r) b_lm(r_hat) with the 24 real
  harmonics of ``cal_blm_ij`` (:816-838), q_nl = sum_m C3B s^2 and the 4-body / 5-body invariants
  (``cal_feat_multi_body`` :745-814); feature order [2-body n] + [l=1 all n, ..., l=4 all n,
  4-body all n, 5-body all n].
* ``nep_eval``: ``NEP.forward`` on CPU (nep_net.py:293-438): feats * q_scaler -> one
  ``FittingNet`` per element (src/model/nep_fitting.py:136-160), Etot per frame, dE/dRi by
  autograd with Ri = (r, x, y, z) as the leaf, forces and virial as ``calculate_force_virial``'s
  CPU branch (nep_net.py:486-560): contraction with Ri_d (Ri_d[0][a] = x_a / r, Ri_d[1+a][a] = 1),
  scatter to the neighbors, upper-triangle virial mirrored, both negated.
* ``zbl_energy``: the ZBL term of ``NEP.calculate_zbl`` / ``cal_zbl`` (nep_net.py:916-991),
  added to Ei when the model's ``zbl`` (outer cutoff) is set and some angular pair lies in
  (0, zbl) (nep_net.py:399-408); its forces follow from the same autograd leaf.
"""
import ctypes
import math
from typing import Dict

import numpy as np
import torch

from . import build as _build

# descriptor constants of nep_net.py:230-242 (C3B with the factor 2 of m > 0 folded in)
C3B = [0.238732414637843, 0.238732414637843, 0.238732414637843,
       0.099471839432435, 1.1936620731892151, 1.1936620731892151, 0.2984155182973038,
       0.2984155182973038,
       0.139260575205408, 0.20889086280811264, 0.20889086280811264, 2.088908628081126,
       2.088908628081126, 0.34815143801352105, 0.34815143801352105,
       0.01119058193614889, 0.44762327744595565, 0.44762327744595565, 0.22381163872297782,
       0.22381163872297782, 3.1333629421216895, 3.1333629421216895, 0.3916703677652112,
       0.3916703677652112]
C4B = [-0.007499480826664, -0.134990654879954, 0.067495327439977, 0.404971964639861,
       -0.809943929279723]
C5B = [0.026596810706114, 0.053193621412227, 0.026596810706114]
L_SLICES = [(0, 3), (3, 8), (8, 15), (15, 24)]

# ZBL universal screening function (Ziegler, Biersack, Littmark) as nep_net.py:222-224 holds it
ZBL_K = 14.399645            # e^2 / (4 pi eps0) in eV A
ZBL_PARA = [0.18175, 3.1998, 0.50986, 0.94229, 0.28022, 0.4029, 0.02817, 0.20162]

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
        P = ctypes.c_void_p
        f = _lib.oracle_nep_neighbor
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int64, P, P, P, P, P, ctypes.c_double, ctypes.c_double,
                      ctypes.c_int64, ctypes.c_int64, ctypes.c_int, P, P, P, P, P, P]
        g = _lib.oracle_nep_maxneigh
        g.restype = None
        g.argtypes = [ctypes.c_int64, P, P, P, P, P, ctypes.c_double, ctypes.c_double,
                      ctypes.c_int64, ctypes.c_int, P, P, P]
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class NeighborOverflow(RuntimeError):
    pass


def neighbor(frames, rc_r: float, rc_a: float, max_r: int, max_a: int, with_rij: bool = True):
    """(NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a) in the order ``calculate_neighbor`` returns them."""
    lib = _load()
    N = frames.natoms
    w = 4 if with_rij else 3
    na, bx, bo, nc, pos = (_c(frames.num_atom, np.int64), _c(frames.box, np.float64),
                           _c(frames.box_orig, np.float64), _c(frames.num_cell, np.int64),
                           _c(frames.position, np.float64))
    NN_r = np.zeros(N, np.int64)
    NN_a = np.zeros(N, np.int64)
    NL_r = np.empty((N, max_r), np.int64)
    NL_a = np.empty((N, max_a), np.int64)
    Ri_r = np.empty((N, max_r, w), np.float64)
    Ri_a = np.empty((N, max_a, w), np.float64)
    ov = lib.oracle_nep_neighbor(frames.nframes, _ptr(na), _ptr(bx), _ptr(bo), _ptr(nc), _ptr(pos),
                                 rc_r, rc_a, max_r, max_a, int(with_rij), _ptr(NN_r), _ptr(NL_r),
                                 _ptr(Ri_r), _ptr(NN_a), _ptr(NL_a), _ptr(Ri_a))
    if ov:
        raise NeighborOverflow(f"max_NN too small: radial {NN_r.max()} / {max_r}, "
                               f"angular {NN_a.max()} / {max_a}")
    return NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a


def maxneigh(frames, rc_r: float, rc_a: float, ntypes: int = 0, with_type: bool = False):
    lib = _load()
    N = frames.natoms
    nt = ntypes if with_type else 1
    NN_r = np.zeros(N * nt, np.int64)
    NN_a = np.zeros(N * nt, np.int64)
    tm = _c(frames.type_map, np.int64)
    lib.oracle_nep_maxneigh(frames.nframes, _ptr(_c(frames.num_atom, np.int64)),
                            _ptr(_c(frames.box, np.float64)), _ptr(_c(frames.box_orig, np.float64)),
                            _ptr(_c(frames.num_cell, np.int64)),
                            _ptr(_c(frames.position, np.float64)), rc_r, rc_a, ntypes,
                            int(with_type), _ptr(tm), _ptr(NN_r), _ptr(NN_a))
    return NN_r, NN_a


# ----------------------------------------------------------------------------------------------
# descriptor and energy
# ----------------------------------------------------------------------------------------------
def _fk(r: torch.Tensor, nk: int, rc: float) -> torch.Tensor:
    """[..., nk] basis f_k(r) = 0.5 (T_k(x) + 1) fc(r), x = 2 (r/rc - 1)^2 - 1, zero outside
    (1e-5, rc]."""
    mask = (r.abs() > 1e-5) & (r <= rc)
    fc = torch.where(mask, 0.5 + 0.5 * torch.cos(np.pi * r / rc), torch.zeros_like(r))
    x = torch.where(mask, 2.0 * (r / rc - 1.0) ** 2 - 1.0, torch.zeros_like(r))
    t = [torch.ones_like(r), x]
    for k in range(2, nk):
        t.append(2.0 * x * t[k - 1] - t[k - 2])
    f = torch.stack([0.5 * (t[k] + 1.0) * fc for k in range(nk)], -1)
    return f * mask.unsqueeze(-1)


def _blm(r: torch.Tensor, xyz: torch.Tensor, rc: float) -> torch.Tensor:
    """[..., 24] real solid-harmonic polynomials of the unit vector (l = 1..4)."""
    mask = (r.abs() > 1e-5) & (r <= rc)
    rinv = torch.where(mask, 1.0 / torch.where(mask, r, torch.ones_like(r)), torch.zeros_like(r))
    x, y, z = (xyz[..., a] * rinv for a in range(3))
    x2, y2, z2 = x * x, y * y, z * z
    d = x2 - y2
    b = [z, x, y,
         3.0 * z2 - 1.0, x * z, y * z, d, 2.0 * x * y,
         (5.0 * z2 - 3.0) * z, (5.0 * z2 - 1.0) * x, (5.0 * z2 - 1.0) * y, d * z, 2.0 * x * y * z,
         (x2 - 3.0 * y2) * x, (3.0 * x2 - y2) * y,
         (35.0 * z2 - 30.0) * z2 + 3.0, (7.0 * z2 - 3.0) * x * z, (7.0 * z2 - 3.0) * y * z,
         (7.0 * z2 - 1.0) * d, (7.0 * z2 - 1.0) * x * y * 2.0, (x2 - 3.0 * y2) * x * z,
         (3.0 * x2 - y2) * y * z, d * d - 4.0 * x2 * y2, 4.0 * x * y * d]
    return torch.stack(b, -1) * mask.unsqueeze(-1)


def _pair_c(c: torch.Tensor, ti: torch.Tensor, NL: torch.Tensor, type_map: torch.Tensor):
    """[N, S, n, k] coefficients c[t_i, t_j] of every slot (zeros for empty slots)."""
    valid = NL >= 0
    tj = type_map[torch.where(valid, NL, torch.zeros_like(NL))]
    cc = c[ti.unsqueeze(1).expand_as(NL), tj]
    return cc * valid[..., None, None]


def features_2b(cfg, c2, type_map, NL_r, Ri_r):
    """[N, n_r] radial descriptor (cal_feat_2body, nep_net.py:717-743)."""
    ti = type_map.long()
    fk = _fk(Ri_r[..., 0], cfg.kr, cfg.cutoff[0])                          # [N, S, k]
    cc = _pair_c(c2, ti, NL_r.long(), type_map.long())                     # [N, S, n, k]
    return torch.einsum("isnk,isk->in", cc, fk)


def features_mb(cfg, c3, type_map, NL_a, Ri_a):
    """[N, F_mb] 3-/4-/5-body descriptor (cal_feat_multi_body, nep_net.py:745-814): l-major
    3-body block, then the 4-body and the 5-body n blocks."""
    ti = type_map.long()
    fk = _fk(Ri_a[..., 0], cfg.ka, cfg.cutoff[1])
    cc = _pair_c(c3, ti, NL_a.long(), type_map.long())
    g = torch.einsum("isnk,isk->isn", cc, fk)                               # [N, S, n]
    b = _blm(Ri_a[..., 0], Ri_a[..., 1:], cfg.cutoff[1])                    # [N, S, 24]
    s = torch.einsum("isn,isl->inl", g, b)                                  # [N, n, 24]
    sq = s * s
    cq = sq * torch.tensor(C3B, dtype=s.dtype)
    qnl = torch.stack([cq[..., a:b_].sum(-1) for a, b_ in L_SLICES[:cfg.l_max[0]]], 1)
    out = [qnl.reshape(qnl.shape[0], -1)]                                   # l-major, then n
    if cfg.l_max[1] > 0:
        s3, s4, s5, s6, s7 = (s[..., k] for k in range(3, 8))
        out.append(C4B[0] * s3 * sq[..., 3] + C4B[1] * s3 * (sq[..., 4] + sq[..., 5])
                   + C4B[2] * s3 * (sq[..., 6] + sq[..., 7])
                   + C4B[3] * s6 * (sq[..., 5] - sq[..., 4]) + C4B[4] * s4 * s5 * s7)
    if cfg.l_max[2] > 0:
        a0, a12 = sq[..., 0], sq[..., 1] + sq[..., 2]
        out.append(C5B[0] * a0 * a0 + C5B[1] * a0 * a12 + C5B[2] * a12 * a12)
    return torch.cat(out, -1)


def features(cfg, p: Dict[str, torch.Tensor], type_map, NL_r, Ri_r, NL_a, Ri_a):
    """[N, F] descriptor q (before q_scaler)."""
    out = []
    if cfg.train_2b:
        out.append(features_2b(cfg, p["c_param_2"], type_map, NL_r, Ri_r))
    if cfg.l_max[0] > 0:
        out.append(features_mb(cfg, p["c_param_3"], type_map, NL_a, Ri_a))
    return torch.cat(out, -1)


def fitting(cfg, p, type_map, feats_in):
    """Ei [N] from the per-element single-hidden-layer nets."""
    Ei = torch.zeros(feats_in.shape[0], dtype=feats_in.dtype)
    for t in range(cfg.ntypes):
        idx = torch.nonzero(type_map.long() == t).flatten()
        if idx.numel() == 0:
            continue
        pre = f"fitting_net.{t}.layers."
        h = torch.tanh(feats_in[idx] @ p[pre + "0.weight"] + p[pre + "0.bias"])
        e = h @ p[pre + "1.weight"] + p[pre + "1.bias"]
        Ei = Ei.index_put((idx,), e.squeeze(-1))
    return Ei


def _ri_d(Ri):
    """[N, S, 4, 3] d(r, x, y, z)/d(x, y, z) for non-empty slots (|r| > 1e-5)."""
    mask = Ri[..., 0].abs() > 1e-5
    d = torch.zeros(*Ri.shape[:2], 4, 3, dtype=Ri.dtype)
    safe = torch.where(mask, Ri[..., 0], torch.ones_like(Ri[..., 0]))
    for a in range(3):
        d[..., 0, a] = torch.where(mask, Ri[..., 1 + a] / safe, torch.zeros_like(safe))
        d[..., 1 + a, a] = mask.to(Ri.dtype)
    return d


def _force_virial(dE, Ri, NL, num_atom):
    """Force gradient and virial of one list, the CPU branch of calculate_force_virial."""
    N = Ri.shape[0]
    dERd = (dE.unsqueeze(-1) * _ri_d(Ri)).sum(-2)                          # [N, S, 3]
    F = torch.zeros(N + 1, 3, dtype=Ri.dtype)
    F[1:] = -dERd.sum(-2)
    idx = (NL.long() + 1).reshape(-1, 1).expand(-1, 3)
    F = F.scatter_add(0, idx, dERd.reshape(-1, 3))
    off = np.concatenate([[0], np.cumsum(num_atom)])
    V = torch.zeros(len(num_atom), 9, dtype=Ri.dtype)
    for b in range(len(num_atom)):
        r = Ri[off[b]:off[b + 1]]
        f = dERd[off[b]:off[b + 1]]
        for (a, c) in [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]:
            V[b, a * 3 + c] = (r[..., 1 + a] * f[..., c]).sum()
        V[b, 3], V[b, 6], V[b, 7] = V[b, 1], V[b, 2], V[b, 5]
    return F[1:], V


def zbl_energy(cfg, type_map, NL_a, Ra, factors: str = "torch"):
    """Ei_zbl [N] (differentiable in Ra) following cal_zbl (nep_net.py:957-991) on the
    angular list restricted to r <= zbl (calculate_zbl :916-955), or None when no pair lies in
    (0, zbl) (the gate of nep_net.py:399-402).

    factors "torch": the element factors exactly as the reference forms them - Z**0.23 and
    K * Z_i * Z_j of int64 element numbers under torch's default float32 dtype, pair by pair in
    the masked order.  torch's float32 pow is not correctly rounded everywhere and its result
    depends on where an element sits in the tensor (vectorised body or scalar tail; Z = 72 gives
    both 2.6741543 and 2.6741545 in one call on x86), so this mode pins the reference bit for
    bit only on the reference's own layout.  factors "rounded": the correctly rounded float32
    Z^0.23, float32 sums and products per element pair - the values the GPU kernel uses."""
    if cfg.zbl is None:
        return None
    rc = float(cfg.zbl) / 2
    r_all = Ra[:, :, 0]
    if not bool(((r_all > 0) & (r_all < cfg.zbl)).any()):
        return None
    keep = (r_all <= cfg.zbl) & (torch.as_tensor(NL_a) != -1)
    r = torch.where(keep, r_all, torch.zeros_like(r_all))
    Z = torch.tensor(list(cfg.atom_type), dtype=torch.int64)
    tm = torch.as_tensor(type_map).long()
    tj = torch.where(keep, tm[torch.as_tensor(NL_a).clamp(min=0)], torch.zeros_like(tm[:1]))
    zi = Z[tm].unsqueeze(1).expand_as(tj)[keep]
    zj = Z[tj][keep]
    rk = r[keep]
    fc = torch.ones_like(rk)
    mid = (rk.abs() >= rc) & (rk <= 2 * rc)
    fc = torch.where(mid, 0.5 + 0.5 * torch.cos((math.pi / rc) * (rk - rc)), fc)
    fc = torch.where(rk.abs() < rc, torch.ones_like(rk), fc)
    if factors == "torch":
        x = rk * (zi ** 0.23 + zj ** 0.23) * 2.134563
        c = ZBL_K * zi * zj
    else:
        Zn = np.array(list(cfg.atom_type), dtype=np.float64)
        f = (Zn ** np.float64(np.float32(0.23))).astype(np.float32)
        Zf = Zn.astype(np.float32)
        s_tab = torch.tensor((f.reshape(-1, 1) + f.reshape(1, -1)).astype(np.float64))
        c_tab = torch.tensor(((np.float32(ZBL_K) * Zf.reshape(-1, 1)) * Zf.reshape(1, -1))
                             .astype(np.float64))
        ti_k = tm.unsqueeze(1).expand_as(tj)[keep]
        tj_k = tj[keep]
        x = rk * s_tab[ti_k, tj_k] * 2.134563
        c = c_tab[ti_k, tj_k]
    phi = ZBL_PARA[0] * torch.exp(-ZBL_PARA[1] * x) + ZBL_PARA[2] * torch.exp(-ZBL_PARA[3] * x) + \
        ZBL_PARA[4] * torch.exp(-ZBL_PARA[5] * x) + ZBL_PARA[6] * torch.exp(-ZBL_PARA[7] * x)
    e = c * phi * fc / rk
    full = torch.zeros(r.shape, dtype=e.dtype)
    full = full.masked_scatter(keep, e)
    return 0.5 * full.sum(-1)


def nep_eval(cfg, p: Dict[str, torch.Tensor], num_atom, type_map, NL_r, Ri_r, NL_a, Ri_a,
             return_feats: bool = False, zbl_factors: str = "torch"):
    """Etot [B, 1], Ei [N], Force [N, 3], Virial [B, 9] (physical force and virial, i.e. the
    values ``NEP.forward`` returns); ``zbl_factors`` as in ``zbl_energy``."""
    num_atom = np.asarray(num_atom).reshape(-1)
    type_map = torch.as_tensor(type_map)
    NL_r, NL_a = torch.as_tensor(NL_r), torch.as_tensor(NL_a)
    Rr = torch.as_tensor(Ri_r, dtype=torch.float64).clone().requires_grad_()
    Ra = torch.as_tensor(Ri_a, dtype=torch.float64).clone().requires_grad_()
    feats = features(cfg, p, type_map, NL_r, Rr, NL_a, Ra)
    Ei = fitting(cfg, p, type_map, feats * p["q_scaler"])
    ez = zbl_energy(cfg, type_map, NL_a, Ra, zbl_factors)
    if ez is not None:
        Ei = Ei + ez
    Etot = torch.stack([e.sum() for e in Ei.split(num_atom.tolist())]).unsqueeze(-1)
    leaves = ([Rr] if cfg.train_2b else []) + ([Ra] if (cfg.l_max[0] > 0 or ez is not None) else [])
    grads = torch.autograd.grad(Etot.sum(), leaves, allow_unused=True)
    F = torch.zeros(Ei.shape[0], 3, dtype=torch.float64)
    V = torch.zeros(len(num_atom), 9, dtype=torch.float64)
    gi = 0
    for R, NL, on in ((Rr, NL_r, cfg.train_2b), (Ra, NL_a, cfg.l_max[0] > 0 or ez is not None)):
        if not on:
            continue
        g = grads[gi]
        gi += 1
        if g is None:
            continue
        f, v = _force_virial(g.detach(), R.detach(), NL, num_atom)
        F, V = F + f, V + v
    out = {"Etot": Etot.detach(), "Ei": Ei.detach(), "Force": -F, "Virial": -V}
    if return_feats:
        out["feats"] = feats.detach()
    return out


TRAIN_KEYS = ("c_param_2", "c_param_3")


def train_grads(cfg, p: Dict[str, torch.Tensor], num_atom, type_map, NL_r, Ri_r, NL_a, Ri_a,
                gE, gF, gV=None):
    """Parameter gradient of L = sum gE Etot + sum gF Force + sum gV Virial (Force, Virial the
    physical values NEP.forward returns) through the CPU branch of NEP.forward with second-order
    autograd, as loss.backward() sees it in training (nep_net.py:293-648).  Returns
    {name: grad} for the descriptor coefficients and every fitting-net tensor."""
    num_atom = np.asarray(num_atom).reshape(-1)
    type_map = torch.as_tensor(type_map)
    NL_r, NL_a = torch.as_tensor(NL_r), torch.as_tensor(NL_a)
    names = [k for k in p if k != "q_scaler"]
    pp = {k: (p[k].detach().clone().requires_grad_() if k in names else p[k]) for k in p}
    Rr = torch.as_tensor(Ri_r, dtype=torch.float64).clone().requires_grad_()
    Ra = torch.as_tensor(Ri_a, dtype=torch.float64).clone().requires_grad_()
    feats = features(cfg, pp, type_map, NL_r, Rr, NL_a, Ra)
    Ei = fitting(cfg, pp, type_map, feats * pp["q_scaler"])
    Etot = torch.stack([e.sum() for e in Ei.split(num_atom.tolist())]).unsqueeze(-1)
    leaves, lists = [], []
    if cfg.train_2b:
        leaves.append(Rr)
        lists.append((Rr, NL_r))
    if cfg.l_max[0] > 0:
        leaves.append(Ra)
        lists.append((Ra, NL_a))
    grads = torch.autograd.grad(Etot.sum(), leaves, create_graph=True, allow_unused=True)
    F = torch.zeros(Ei.shape[0], 3, dtype=torch.float64)
    V = torch.zeros(len(num_atom), 9, dtype=torch.float64)
    for g, (R, NL) in zip(grads, lists):
        if g is None:
            continue
        f, v = _force_virial(g, R.detach(), NL, num_atom)
        F, V = F + f, V + v
    L = (torch.as_tensor(gE) * Etot.reshape(-1)).sum() + (torch.as_tensor(gF) * -F).sum()
    if gV is not None:
        L = L + (torch.as_tensor(gV) * -V).sum()
    leaves_p = [pp[k] for k in names]
    gs = torch.autograd.grad(L, leaves_p, allow_unused=True)
    return {k: (torch.zeros_like(pp[k]) if g is None else g.detach()) for k, g in zip(names, gs)}
