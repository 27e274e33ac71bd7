"""Drop-ins for MatPL's NEP training operators: ``CalcOps.calculateNepFeat`` /
``calculateNepMbFeat`` (descriptor with first and second backward, src/op/src/CalcOps.cpp:385-1023)
and ``calculateNepForce`` / ``calculateNepVirial`` (CalcOps.cpp:75-330), with the reference's
signatures and list returns, as ``nep_net.NEP.forward`` calls them (nep_net.py:352-380, 612-631).

The descriptor functions run ``matpl_nep_feat_op`` (csrc/nep_train.cu).  Like the reference's
``CalculateNepFeat``: backward gives dL/dc and dL/dRi; the Grad function's own backward gives
dL/dG and dL/dc from the gradient reaching dL/dRi (the force-loss path of training); the
gradient reaching dL/dc of the Grad function is not propagated further (the reference returns
none for it either), nor is a third-order term in Ri.  dL/dRi holds the partial derivatives in
the four columns (r, x, y, z) taken as independent, as the reference's CPU descriptor gives them
under autograd; the reference's CUDA kernel distributes the angular part between the columns in
GPUMD's way, and both give the same forces once contracted with Ri_d.  The force and virial
functions reuse the DP force / virial kernels (one configuration of N atoms); the virial is
summed per image of ``num_atom`` and its backward uses each image's own gradient (the
reference's CUDA backward applies the first image's to all atoms).

For ``nep_train.NEPTrain`` the module also has the training step's own forms: ``nep_feat_d12``
(the descriptor's d12 gradient alone, the force path), the c-gradient reduction
``matpl_nep_cgrad`` behind every backward, ``nep_force_virial`` (forces and per-image virial
from dE and the (r, x, y, z) rows, calculate_Ri formed in the kernel) and ``nep_zbl`` (the ZBL
term, nep_net.py:916-991).
"""
from typing import List

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr
from .ops import _CalculateForce, _dtype_code, _require_cuda, _stream

PART_RADIAL, PART_ANGULAR = 0, 1
MODE_FWD, MODE_BWD, MODE_BWD2 = 0, 1, 2

_check_each_call = True
_err_words = {}


def set_check_errors(each_call: bool):
    """True (default): every descriptor call reads the kernels' error word (one device sync).
    False: the word accumulates on the device until ``check_errors()`` (training loops)."""
    global _check_each_call
    _check_each_call = bool(each_call)


def _err_word(dev):
    w = _err_words.get(dev)
    if w is None:
        w = torch.zeros(1, dtype=torch.int32, device=dev)
        _err_words[dev] = w
    return w


def check_errors(device=None):
    """Raise if a descriptor kernel flagged an error since the last check (then clear it)."""
    for dev, w in list(_err_words.items()):
        if device is not None and dev != torch.device(device):
            continue
        code = int(w.item())
        if code:
            w.zero_()
            raise _lib.MatplError(f"matpl_nep_feat_op kernel error {code} (2 = bad type, "
                                  "5 = list index outside the atoms)")


def _nfeat(part, nmax, l3, l4, l5):
    if part == PART_RADIAL:
        return nmax
    return nmax * (l3 + (1 if l4 > 0 else 0) + (1 if l5 > 0 else 0))


@_lib.on_device
def _feat_call(part, mode, coeff, d12, NL, atom_map, rc, l3=0, l4=0, l5=0, G=None, H=None,
               want_d=True, want_c=True):
    """One launch of ``matpl_nep_feat_op``; returns (q or gso, grad_d12, W).  In the backward
    mode ``want_d`` / ``want_c`` select grad_d12 and the c-gradient table (None if not)."""
    _require_cuda(coeff, d12, NL, atom_map)
    N, NN = NL.shape
    T, _, nmax, K = coeff.shape
    dev, dt = d12.device, d12.dtype
    code = _dtype_code(d12)
    c = coeff.detach().to(dt).contiguous()
    dd = d12.detach().contiguous()
    nl = NL.contiguous().to(torch.int64)
    tm = atom_map.contiguous().to(torch.int64)
    F = _nfeat(part, nmax, l3, l4, l5)
    err = _err_word(dev)
    q = gd = W = None
    Gc = G.detach().to(dt).contiguous() if G is not None else None
    Hc = H.detach().to(dt).contiguous() if H is not None else None
    if mode in (MODE_FWD, MODE_BWD2):
        q = torch.empty(N, F, dtype=dt, device=dev) if mode == MODE_FWD else \
            torch.zeros(N, F, dtype=dt, device=dev)
        if N * NN == 0:
            q.zero_()
    if mode == MODE_BWD and want_d:
        gd = torch.zeros(N, NN, 4, dtype=dt, device=dev)
    if mode == MODE_BWD2 or (mode == MODE_BWD and want_c):
        shape = (N, T, K) if part == PART_RADIAL else (N, T, nmax, K)
        W = torch.zeros(shape, dtype=dt, device=dev)
    check(_lib.load().matpl_nep_feat_op(
        code, part, mode, N, NN, T, nmax, K, l3, l4, l5, float(rc), ptr(c), ptr(dd), ptr(nl),
        ptr(tm), ptr(Gc), F, ptr(Hc), ptr(q), F, ptr(gd), ptr(W), ptr(err), _stream(dev)),
        "matpl_nep_feat_op")
    if _check_each_call:
        check_errors(dev)
    return q, gd, W


@_lib.on_device
def _c_grad(part, W, G, atom_map, T):
    """dL/dc [T, T, n, K] from the per-atom tables (``matpl_nep_cgrad``): radial
    sum_i G[i, n] W[i, t, k]; angular sum_i W[i] (G already folded in), each into row t_i."""
    dev, dt = W.device, W.dtype
    N = W.shape[0]
    if part == PART_RADIAL:
        _, Tt, K = W.shape
        Gc = G.detach().to(dt).contiguous()
        n = Gc.shape[1]
    else:
        _, Tt, n, K = W.shape
        Gc = None
    out = torch.empty(T, Tt, n, K, dtype=dt, device=dev)
    tm = atom_map.contiguous().to(torch.int64)
    check(_lib.load().matpl_nep_cgrad(_dtype_code(W), part, N, T, n, K, ptr(tm), ptr(Gc),
                                      n, ptr(W.contiguous()), ptr(out), ptr(_err_word(dev)),
                                      _stream(dev)), "matpl_nep_cgrad")
    return out


def _second_backward(ctx, g_gd):
    """Gradients (G, coeff) of grad_d12 = G . dq/dd12 for its upstream gradient g_gd: the
    second backward mode (gso = dq/dd12 . g_gd, and the c-terms)."""
    G, coeff, d12, NL, atom_map = ctx.saved_tensors
    part, rc, l3, l4, l5 = ctx.meta
    gso, _, W2 = _feat_call(part, MODE_BWD2, coeff, d12, NL, atom_map, rc, l3, l4, l5,
                            G=G, H=g_gd)
    gsc = _c_grad(part, W2, G.detach(), atom_map, coeff.shape[0]).to(coeff.dtype)
    return gso.to(G.dtype), gsc


class _NepFeatGrad(torch.autograd.Function):
    """(dL/dc, grad_d12) of the features for G = dL/dq; differentiable in G and c."""

    @staticmethod
    def forward(ctx, G, coeff, d12, NL, atom_map, part, rc, l3, l4, l5):
        _, gd, W = _feat_call(part, MODE_BWD, coeff, d12, NL, atom_map, rc, l3, l4, l5, G=G)
        gc = _c_grad(part, W, G.detach(), atom_map, coeff.shape[0]).to(coeff.dtype)
        ctx.save_for_backward(G, coeff, d12, NL, atom_map)
        ctx.meta = (part, rc, l3, l4, l5)
        return gc, gd

    @staticmethod
    def backward(ctx, g_gc, g_gd):
        if g_gd is None:
            return (None,) * 10
        gso, gsc = _second_backward(ctx, g_gd)
        return gso, gsc, None, None, None, None, None, None, None, None


class _NepFeatD12(torch.autograd.Function):
    """grad_d12 = G . dq/dd12 alone (the force path); differentiable in G and c."""

    @staticmethod
    def forward(ctx, G, coeff, d12, NL, atom_map, part, rc, l3, l4, l5):
        _, gd, _ = _feat_call(part, MODE_BWD, coeff, d12, NL, atom_map, rc, l3, l4, l5, G=G,
                              want_c=False)
        ctx.save_for_backward(G, coeff, d12, NL, atom_map)
        ctx.meta = (part, rc, l3, l4, l5)
        return gd

    @staticmethod
    def backward(ctx, g_gd):
        gso, gsc = _second_backward(ctx, g_gd)
        return gso, gsc, None, None, None, None, None, None, None, None


class _NepFeatCGrad(torch.autograd.Function):
    """dL/dc alone for G = dL/dq (the features' backward when d12 needs no gradient)."""

    @staticmethod
    def forward(ctx, G, coeff, d12, NL, atom_map, part, rc, l3, l4, l5):
        _, _, W = _feat_call(part, MODE_BWD, coeff, d12, NL, atom_map, rc, l3, l4, l5, G=G,
                             want_d=False)
        return _c_grad(part, W, G.detach(), atom_map, coeff.shape[0]).to(coeff.dtype)

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, g):
        raise RuntimeError("the coefficient gradient of a descriptor whose d12 needs no "
                           "gradient is not differentiable again")


class _NepFeat(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coeff, d12, NL, atom_map, part, rc, l3, l4, l5):
        q, _, _ = _feat_call(part, MODE_FWD, coeff, d12, NL, atom_map, rc, l3, l4, l5)
        ctx.save_for_backward(coeff, d12, NL, atom_map)
        ctx.meta = (part, rc, l3, l4, l5)
        return q

    @staticmethod
    def backward(ctx, gq):
        coeff, d12, NL, atom_map = ctx.saved_tensors
        part, rc, l3, l4, l5 = ctx.meta
        if not ctx.needs_input_grad[1]:
            gc = _NepFeatCGrad.apply(gq, coeff, d12, NL, atom_map, part, rc, l3, l4, l5)
            return gc, None, None, None, None, None, None, None, None
        gc, gd = _NepFeatGrad.apply(gq, coeff, d12, NL, atom_map, part, rc, l3, l4, l5)
        return gc, gd, None, None, None, None, None, None, None


def nep_feat_d12(coeff: torch.Tensor, G: torch.Tensor, d12: torch.Tensor, NL: torch.Tensor,
                 atom_map: torch.Tensor, angular: bool, rc: float, lmax_3: int = 0,
                 lmax_4: int = 0, lmax_5: int = 0) -> torch.Tensor:
    """grad_d12 [N, NN, 4] = G . dq/dd12 of one list's features for G = dE/dq [N, F] (the
    gradient the force path of NEP.forward takes of the descriptor, nep_net.py:603-611),
    without the coefficient table; differentiable in G and coeff (second backward mode)."""
    part = PART_ANGULAR if angular else PART_RADIAL
    return _NepFeatD12.apply(G, coeff, d12, NL, atom_map, part, float(rc), int(lmax_3),
                             int(lmax_4), int(lmax_5))


def calculateNepFeat(coeff2: torch.Tensor, d12_radial: torch.Tensor, NL_radial: torch.Tensor,
                     atom_map: torch.Tensor, feats: torch.Tensor, rcut_radial: float,
                     multi_feat_num: int) -> List[torch.Tensor]:
    """``CalcOps.calculateNepFeat`` (CalcOps.cpp:385-680): coeff2 [T, T, n, K], d12_radial
    [N, NN, 4] (r, x, y, z), NL_radial [N, NN] int64 (-1 empty), atom_map [N] -> [feat_2b
    [N, n]].  ``feats`` (the reference's zero-filled output buffer) only fixes the dtype;
    ``multi_feat_num`` is accepted for the signature."""
    return [_NepFeat.apply(coeff2, d12_radial, NL_radial, atom_map, PART_RADIAL,
                           float(rcut_radial), 0, 0, 0).to(feats.dtype)]


def calculateNepMbFeat(coeff3: torch.Tensor, d12: torch.Tensor, NL: torch.Tensor,
                       atom_map: torch.Tensor, feats: torch.Tensor, feat_2b_num: int,
                       lmax_3: int, lmax_4: int, lmax_5: int,
                       rcut_angular: float) -> List[torch.Tensor]:
    """``CalcOps.calculateNepMbFeat`` (CalcOps.cpp:680-1023) -> [feat_mb [N, n*(l3 + 4b + 5b)]]
    in the order l-major 3-body, 4-body, 5-body."""
    return [_NepFeat.apply(coeff3, d12, NL, atom_map, PART_ANGULAR, float(rcut_angular),
                           int(lmax_3), int(lmax_4), int(lmax_5)).to(feats.dtype)]


def calculateNepForce(list_neigh: torch.Tensor, dE: torch.Tensor, Ri_d: torch.Tensor,
                      F: torch.Tensor) -> List[torch.Tensor]:
    """``CalcOps.calculateNepForce`` (CalcOps.cpp:75-168): list_neigh [N, NN] int64 (-1 empty),
    dE [N, NN, 4], Ri_d [N, NN*4, 3] (or [N, NN, 4, 3]), F [N, 3] the centre term -> [F plus
    the neighbors' terms]; differentiable in dE (centre and neighbor parts)."""
    _require_cuda(list_neigh, dE, Ri_d, F)
    N, NN = list_neigh.shape
    out = _CalculateForce.apply(list_neigh.reshape(1, N, NN), dE.reshape(1, N, 4 * NN),
                                Ri_d.reshape(1, N, 4 * NN, 3), F.reshape(1, N, 3), 0)
    return [out.reshape(N, 3)]


_img_cache = {}


def _image_index(counts, dev):
    """[N] image of every atom for per-image sums, cached per (counts, device)."""
    key = (counts, dev)
    t = _img_cache.get(key)
    if t is None:
        t = torch.repeat_interleave(torch.arange(len(counts)), torch.tensor(counts)).to(dev)
        if len(_img_cache) > 64:
            _img_cache.clear()
        _img_cache[key] = t
    return t


class _NepForceVirial(torch.autograd.Function):
    """Forces [N, 3] and per-image virial [B, 9] of one list (``matpl_nep_force_virial``);
    linear in dE, its backward (``matpl_nep_force_virial_grad``) is the transpose map."""

    @staticmethod
    @_lib.on_device
    def forward(ctx, NL, dE, Ri, image_of, nimages):
        N, NN = NL.shape
        dev, dt = dE.device, dE.dtype
        nl = NL.contiguous().to(torch.int64)
        R = Ri.detach().to(dt).contiguous()
        F = torch.empty(N, 3, dtype=dt, device=dev)
        V = torch.empty(nimages, 9, dtype=dt, device=dev)
        check(_lib.load().matpl_nep_force_virial(
            _dtype_code(dE), N, NN, nimages, ptr(nl), ptr(image_of), ptr(dE.contiguous()),
            ptr(R), ptr(F), ptr(V), ptr(_err_word(dev)), _stream(dev)), "matpl_nep_force_virial")
        ctx.save_for_backward(nl, R, image_of)
        ctx.nimages = nimages
        return F, V

    @staticmethod
    @torch.autograd.function.once_differentiable
    @_lib.on_device
    def backward(ctx, gF, gV):
        nl, R, image_of = ctx.saved_tensors
        N, NN = nl.shape
        gdE = torch.empty(N, NN, 4, dtype=R.dtype, device=R.device)
        gFc = gF.contiguous().to(R.dtype) if gF is not None else None
        gVc = gV.contiguous().to(R.dtype) if gV is not None else None
        check(_lib.load().matpl_nep_force_virial_grad(
            _dtype_code(R), N, NN, ctx.nimages, ptr(nl), ptr(image_of), ptr(R), ptr(gFc),
            ptr(gVc), ptr(gdE), ptr(_err_word(R.device)), _stream(R.device)),
            "matpl_nep_force_virial_grad")
        return None, gdE, None, None, None


def nep_force_virial(NL: torch.Tensor, dE: torch.Tensor, Ri: torch.Tensor, num_atom
                     ) -> List[torch.Tensor]:
    """[force [N, 3], virial [B, 9]] of one list: calculateNepForce with the centre term
    -sum_s dE . Ri_d and calculateNepVirial's per-image sum, with Ri_d = calculate_Ri(Ri)
    formed in the kernel (frames contiguous with sizes ``num_atom``); differentiable in dE."""
    _require_cuda(NL, dE, Ri)
    counts = tuple(int(c) for c in np.asarray(num_atom).reshape(-1)) \
        if not torch.is_tensor(num_atom) else tuple(int(c) for c in num_atom.reshape(-1).tolist())
    img = _image_index(counts, dE.device)
    F, V = _NepForceVirial.apply(NL, dE, Ri, img, len(counts))
    return [F, V]


ZBL_K = 14.399645       # e^2 / (4 pi eps0) in eV A, nep_net.py:223
_zbl_tables = {}


def zbl_tables(atom_type, dev):
    """(pair_s, pair_c) [T, T] f64 on dev: Z_i^0.23 + Z_j^0.23 and K Z_i Z_j in float32 as
    cal_zbl (nep_net.py:985-989) forms them under torch's default float32 dtype: the powers
    rounded to float32, their sum and the products rounded in float32.  Z^0.23 is taken as the
    correctly rounded float32 value (float64 pow, then rounded): torch's own float32 pow, which
    the reference calls, is not correctly rounded everywhere and depends on where an element
    sits in the tensor (on x86 one call gives 2.6741543 and 2.6741545 for Z = 72, and one ulp off
    for Z = 98, 101-103, 110, 115, 116 in an arange), so no fixed table reproduces it pair for
    pair.  Cached per (elements, device)."""
    key = (tuple(int(z) for z in atom_type), dev)
    t = _zbl_tables.get(key)
    if t is None:
        Z = np.array(key[0], dtype=np.float64)
        f = (Z ** np.float64(np.float32(0.23))).astype(np.float32)
        s = f.reshape(-1, 1) + f.reshape(1, -1)                          # float32 adds
        Zf = Z.astype(np.float32)
        c = (np.float32(ZBL_K) * Zf.reshape(-1, 1)) * Zf.reshape(1, -1)   # float32 products
        t = (torch.tensor(s.astype(np.float64), device=dev),
             torch.tensor(c.astype(np.float64), device=dev))
        _zbl_tables[key] = t
    return t


@_lib.on_device
def nep_zbl(zbl: float, atom_type, NL_a: torch.Tensor, Ri_a: torch.Tensor,
            type_map: torch.Tensor, counts, Ei: torch.Tensor, Etot, force: torch.Tensor,
            virial: torch.Tensor) -> None:
    """Adds the ZBL term (``matpl_nep_zbl``; nep_net.py:399-408, 916-991) of the angular list
    to Ei [N], Etot [B] f64 (or None), force [N, 3] (Ei's dtype) and virial [B, 9] f64 in
    place: per pair 0 < r <= zbl, e = K Z_i Z_j phi(r (Z_i^0.23 + Z_j^0.23) / 0.46848) fc(r) / r,
    half of it to the centre.  Frames contiguous with sizes ``counts``."""
    _require_cuda(NL_a, Ri_a, type_map, Ei, force, virial)
    dev = Ei.device
    N, NN = NL_a.shape
    pair_s, pair_c = zbl_tables(atom_type, dev)
    nl = NL_a.contiguous().to(torch.int64)
    tm = type_map.reshape(-1).contiguous().to(torch.int64)
    R = Ri_a.detach().contiguous()
    if R.dtype != torch.float64 and Ei.dtype == torch.float64:
        R = R.to(torch.float64)
    img = _image_index(tuple(int(c) for c in counts), dev)
    if virial.dtype != torch.float64 or not virial.is_contiguous():
        raise _lib.MatplError("nep_zbl: virial must be a contiguous float64 tensor")
    check(_lib.load().matpl_nep_zbl(
        _dtype_code(Ei), _dtype_code(R), N, NN, len(counts), ptr(nl), ptr(R), ptr(tm), ptr(img),
        len(atom_type), ptr(pair_s), ptr(pair_c), float(zbl), ptr(Ei), ptr(Etot), ptr(force),
        ptr(virial), ptr(_err_word(dev)), _stream(dev)), "matpl_nep_zbl")


class _NepVirial(torch.autograd.Function):
    @staticmethod
    @_lib.on_device
    def forward(ctx, list_neigh, dE, Rij, Ri_d, num_atom):
        N, NN = list_neigh.shape
        nl = list_neigh.contiguous().to(torch.int32)
        dE_c = dE.contiguous().reshape(N, 4 * NN)
        Rj = Rij.contiguous().to(dE.dtype).reshape(N, NN, 3)
        Rd = Ri_d.contiguous().reshape(N, 4 * NN, 3)
        counts = [int(v) for v in np.asarray(num_atom.detach().cpu()).reshape(-1)]
        vir1 = torch.empty(1, 9, dtype=dE.dtype, device=dE.device)
        avir = torch.empty(N, 9, dtype=dE.dtype, device=dE.device)
        check(_lib.load().matpl_calc_virial(_dtype_code(dE), ptr(nl), ptr(dE_c), ptr(Rj), ptr(Rd),
                                            1, N, NN, 0, ptr(vir1), ptr(avir), _stream(dE.device)),
              "matpl_calc_virial")
        img = _image_index(tuple(counts), dE.device)
        vir = torch.zeros(len(counts), 9, dtype=dE.dtype, device=dE.device).index_add_(0, img,
                                                                                       avir)
        ctx.save_for_backward(nl, Rj, Rd)
        ctx.counts = counts
        ctx.dshape = dE.shape
        ctx.mark_non_differentiable(avir)
        return vir, avir

    @staticmethod
    @_lib.on_device
    def backward(ctx, grad_vir, grad_avir):
        nl, Rj, Rd = ctx.saved_tensors
        N, NN = nl.shape
        grad = torch.zeros(N, 4 * NN, dtype=Rd.dtype, device=Rd.device)
        if grad_vir is not None:
            g = grad_vir.contiguous().to(Rd.dtype)
            lib = _lib.load()
            off = 0
            for b, n in enumerate(ctx.counts):
                if n:
                    check(lib.matpl_calc_virial_grad(
                        _dtype_code(Rd), ptr(nl[off:off + n]), ptr(Rj[off:off + n]),
                        ptr(Rd[off:off + n]), ptr(g[b:b + 1]), 1, n, NN, ptr(grad[off:off + n]),
                        _stream(Rd.device)), "matpl_calc_virial_grad")
                off += n
        return None, grad.reshape(ctx.dshape), None, None, None


def calculateNepVirial(list_neigh: torch.Tensor, dE: torch.Tensor, Rij: torch.Tensor,
                       Ri_d: torch.Tensor, num_atom: torch.Tensor) -> List[torch.Tensor]:
    """``CalcOps.calculateNepVirial`` (CalcOps.cpp:239-330) -> [virial [B, 9] per image,
    atom_virial [N, 9]], virial[a*3+c] = sum (dE . Ri_d)_a Rij_c credited to the neighbor."""
    _require_cuda(list_neigh, dE, Rij, Ri_d)
    v, av = _NepVirial.apply(list_neigh, dE, Rij, Ri_d, num_atom)
    return [v, av]
