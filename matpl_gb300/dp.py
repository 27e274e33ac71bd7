"""GB300 DP se_e2_a model with the reference ``DP.forward`` interface.

``DP(cfg, params, davg, dstd).forward(list_neigh, Imagetype_map, atom_type, ImageDR, nghost)``
returns ``(Etot [B,1], Ei [B,n], Force [B,N+nghost,3], Egroup, Virial [B,9])`` exactly like
``src/model/dp_dp.py:167-215`` / ``dp_dp_script.py`` (the TorchScript module LAMMPS calls,
``src/lmps/lammps-libtorch/MATPL/pair_matpl.cpp:932``):

* ``list_neigh`` [B,N,S] int32, 1-based (0 = empty), per-type blocks of ``maxNeighborNum``;
* ``Imagetype_map`` [N] model type index of each atom; ``atom_type`` the image's elements;
* ``Ei`` is returned in the reference's type-grouped order (dp_dp.py:339);
* ``Virial[a*3+c] = sum f_a Rij_c`` (the GPU op convention, calculateVirial.cu:80).

The whole evaluation is one call into ``matpl_dp_eval`` (four kernels, no per-pair HBM
traffic).  Parameters use the reference's state-dict names; ``pack_params`` lays them out as
``csrc/dp_layout.cuh`` expects.
"""
import ctypes
from typing import Dict, List, Optional

import torch

from . import _lib
from ._lib import (MATPL_F32, MATPL_F64, MATPL_MIXED, MATPL_MIXED_FAST, MATPL_MIXED_TANHF,
                   MatplDpModel, check, ptr)

# precision name -> (C ABI compute form, storage dtype)
PRECISIONS = {
    "float64": (MATPL_F64, torch.float64),
    "float32": (MATPL_F32, torch.float32),
    "mixed": (MATPL_MIXED, torch.float32),              # tcgen05 BF16x3 GEMMs, tanh.approx
    "mixed_fast": (MATPL_MIXED_FAST, torch.float32),    # tcgen05 BF16 embedding GEMMs
    "mixed_tanhf": (MATPL_MIXED_TANHF, torch.float32),  # tcgen05 BF16x3 GEMMs, CUDA tanhf
}
from .params import DPConfig

E, M2, DIN, F = 25, 16, 400, 50
EMB_SIZE = 6 * E + 2 * E * E
FIT_W0, FIT_B0 = 0, DIN * F
FIT_W1 = FIT_B0 + F
FIT_B1 = FIT_W1 + F * F
FIT_DT1 = FIT_B1 + F
FIT_W2 = FIT_DT1 + F
FIT_B2 = FIT_W2 + F * F
FIT_DT2 = FIT_B2 + F
FIT_W3 = FIT_DT2 + F
FIT_B3 = FIT_W3 + F
FIT_W0T = FIT_B3 + 4
FIT_W1T = FIT_W0T + F * DIN
FIT_W2T = FIT_W1T + F * F
FIT_SIZE = FIT_W2T + F * F


def check_shape(cfg: DPConfig):
    if list(cfg.emb_sizes) != [E, E, E] or cfg.M2 != M2 or list(cfg.fit_sizes) != [F, F, F, 1]:
        raise _lib.MatplError(
            "compiled DP kernels cover embedding [25,25,25], M2=16, fitting [50,50,50,1]; got "
            f"{cfg.emb_sizes}, M2={cfg.M2}, {cfg.fit_sizes}")


def pack_params(cfg: DPConfig, params: Dict[str, torch.Tensor], dtype=torch.float64) -> torch.Tensor:
    """Flatten reference-named parameters into the packed layout of csrc/dp_layout.cuh."""
    check_shape(cfg)
    nt = cfg.ntypes
    out = torch.zeros(nt * nt * EMB_SIZE + nt * FIT_SIZE, dtype=torch.float64)

    def g(k, shape=None, default=None):
        v = params.get(k)
        if v is None:
            if default is None:
                raise KeyError(k)
            return default
        return v.detach().to(torch.float64).cpu().reshape(-1)

    ones_e, zeros_e = torch.ones(E, dtype=torch.float64), torch.zeros(E, dtype=torch.float64)
    for k in range(nt * nt):
        base = k * EMB_SIZE
        pre = f"embedding_net.{k}.layers."
        parts = [g(pre + "0.weight"), g(pre + "0.bias", default=zeros_e),
                 g(pre + "1.weight"), g(pre + "1.bias", default=zeros_e),
                 g(pre + "1.resnet_dt", default=ones_e),
                 g(pre + "2.weight"), g(pre + "2.bias", default=zeros_e),
                 g(pre + "2.resnet_dt", default=ones_e)]
        flat = torch.cat(parts)
        assert flat.numel() == EMB_SIZE
        out[base:base + EMB_SIZE] = flat
    ones_f, zeros_f = torch.ones(F, dtype=torch.float64), torch.zeros(F, dtype=torch.float64)
    for t in range(nt):
        base = nt * nt * EMB_SIZE + t * FIT_SIZE
        pre = f"fitting_net.{t}.layers."
        W0 = g(pre + "0.weight").reshape(DIN, F)
        W1 = g(pre + "1.weight").reshape(F, F)
        W2 = g(pre + "2.weight").reshape(F, F)
        o = out[base:base + FIT_SIZE]
        o[FIT_W0:FIT_B0] = W0.reshape(-1)
        o[FIT_B0:FIT_W1] = g(pre + "0.bias", default=zeros_f)
        o[FIT_W1:FIT_B1] = W1.reshape(-1)
        o[FIT_B1:FIT_DT1] = g(pre + "1.bias", default=zeros_f)
        o[FIT_DT1:FIT_W2] = g(pre + "1.resnet_dt", default=ones_f)
        o[FIT_W2:FIT_B2] = W2.reshape(-1)
        o[FIT_B2:FIT_DT2] = g(pre + "2.bias", default=zeros_f)
        o[FIT_DT2:FIT_W3] = g(pre + "2.resnet_dt", default=ones_f)
        o[FIT_W3:FIT_B3] = g(pre + "3.weight")
        o[FIT_B3] = g(pre + "3.bias", default=torch.zeros(1, dtype=torch.float64))[0]
        o[FIT_W0T:FIT_W1T] = W0.t().contiguous().reshape(-1)
        o[FIT_W1T:FIT_W2T] = W1.t().contiguous().reshape(-1)
        o[FIT_W2T:FIT_SIZE] = W2.t().contiguous().reshape(-1)
    return out.to(dtype)


def per_type_stats(arr: torch.Tensor, ntypes: int) -> torch.Tensor:
    """[ntypes, S*4] (tiled, as the reference stores davg/dstd) -> [ntypes, 4]."""
    a = arr.detach().to(torch.float64).cpu().reshape(ntypes, -1, 4)
    if not torch.equal(a, a[:, :1, :].expand_as(a)):
        raise _lib.MatplError("davg/dstd must be the same 4-vector for every slot of a centre type "
                              "(the layout dpuni_data_loader.set_davg_dstd produces)")
    return a[:, 0, :].contiguous()


class DP(torch.nn.Module):
    """Inference DP se_e2_a on GB300.

    ``precision``: "float64" | "float32" (plain SIMT forms) | "mixed" | "mixed_fast" |
    "mixed_tanhf" (embedding and fitting GEMMs on the tcgen05 tensor cores, FP32 data, FP64
    energy / virial sums).  ``check_errors`` reads the kernels' error word after every call (one
    device sync); the benchmark turns it off inside its timed loop."""

    def __init__(self, cfg: DPConfig, params: Dict[str, torch.Tensor], davg, dstd,
                 precision: str = "float64", device="cuda", check_errors: bool = True,
                 packed: Optional[torch.Tensor] = None, compress: Optional[Dict] = None):
        super().__init__()
        check_shape(cfg)
        if precision not in PRECISIONS:
            raise _lib.MatplError(f"unknown precision {precision!r}; one of {list(PRECISIONS)}")
        self.cfg = cfg
        self.precision = precision
        self.code, self.dtype = PRECISIONS[precision]
        self.check_errors = check_errors
        dev = torch.device(device)
        self.register_buffer("err", torch.zeros(1, dtype=torch.int32, device=dev))
        self.device = dev
        if packed is None:
            packed = pack_params(cfg, params, self.dtype)
        self.register_buffer("packed", packed.to(device=dev, dtype=self.dtype).clone())
        davg = torch.as_tensor(davg)
        dstd = torch.as_tensor(dstd)
        self.register_buffer("davg4", per_type_stats(davg, cfg.ntypes).to(dev, self.dtype))
        self.register_buffer("dstd4", per_type_stats(dstd, cfg.ntypes).to(dev, self.dtype))
        self._perm_cache = {}
        # compressed model: the tables of compress.build_table (ckpt_compress.py) in the fused
        # kernels instead of the embedding nets
        self.compress = compress
        if compress is not None:
            import numpy as _np
            tab = torch.as_tensor(_np.asarray(compress["table"]))
            if tab.dim() != 4 or tab.shape[0] != cfg.ntypes ** 2 or tab.shape[2] != E:
                raise _lib.MatplError("compress table must be [ntypes^2, rows, 25, order + 1]")
            self.register_buffer("ctable", tab.to(device=dev, dtype=self.dtype).contiguous())
            self._ctab = (int(tab.shape[1]), int(compress["order"]), float(compress["dx"]),
                          float(compress["sij_min"]), float(compress["sij_max"]))

    # dp_dp.py:145-165
    def present_types(self, atom_type) -> List[int]:
        at = [int(a) for a in (atom_type.tolist() if isinstance(atom_type, torch.Tensor) else atom_type)]
        return [self.cfg.atom_type.index(a) for a in at if a in self.cfg.atom_type]

    def _model_struct(self, present: List[int]) -> MatplDpModel:
        m = MatplDpModel()
        m.ntypes = self.cfg.ntypes
        m.m = self.cfg.maxNeighborNum
        m.npresent = len(present)
        for q, t in enumerate(present):
            m.present[q] = t
        m.rmin, m.rmax = float(self.cfg.Rmin), float(self.cfg.Rmax)
        m.params, m.davg, m.dstd = ptr(self.packed), ptr(self.davg4), ptr(self.dstd4)
        m.err_dev = ptr(self.err)
        if self.compress is not None:
            m.ctable = ptr(self.ctable)
            m.ctab_rows, m.ctab_order, m.ctab_dx, m.ctab_smin, m.ctab_smax = self._ctab
        return m

    def _grouped_perm(self, tmap: torch.Tensor, present: List[int]) -> torch.Tensor:
        key = (tmap.data_ptr(), tmap.numel(), tuple(present))
        p = self._perm_cache.get(key)
        if p is None:
            tl = tmap.long()
            p = torch.cat([torch.nonzero(tl == t).flatten() for t in present])
            self._perm_cache = {key: p}
        return p

    @_lib.on_device
    def evaluate(self, list_neigh: torch.Tensor, Imagetype_map: torch.Tensor, present: List[int],
                 ImageDR: torch.Tensor, nghost: int = 0, out: Optional[dict] = None,
                 num_neigh: Optional[torch.Tensor] = None):
        """Raw fused evaluation: returns dict(Ei_atom [B,N], Etot [B] f64, Force, Virial [B,9] f64).

        ``num_neigh`` [B,N,ntypes] int32 (from ``find_neighbore(..., occupied_only=True)``)
        gives the type blocks' lengths; the list's slots past them are then never read."""
        if not (list_neigh.is_cuda and ImageDR.is_cuda):
            raise _lib.MatplError("DP.evaluate takes CUDA tensors (no CPU fallback)")
        B, N, S = list_neigh.shape
        dev = ImageDR.device
        ln = list_neigh if list_neigh.dtype == torch.int32 and list_neigh.is_contiguous() \
            else list_neigh.to(torch.int32).contiguous()
        idr = ImageDR if ImageDR.dtype == self.dtype and ImageDR.is_contiguous() \
            else ImageDR.to(self.dtype).contiguous()
        tm = Imagetype_map if Imagetype_map.dtype == torch.int32 and Imagetype_map.is_cuda \
            else Imagetype_map.to(device=dev, dtype=torch.int32).contiguous()
        if out is None:
            out = {"Ei_atom": torch.empty(B, N, dtype=self.dtype, device=dev),
                   "Etot": torch.empty(B, dtype=torch.float64, device=dev),
                   "Force": torch.empty(B, N + nghost, 3, dtype=self.dtype, device=dev),
                   "Virial": torch.empty(B, 9, dtype=torch.float64, device=dev)}
        lib = _lib.load()
        from .ops import workspace
        nbytes = lib.matpl_dp_workspace_bytes(self.code, B, N)
        ws = workspace(dev, nbytes, "dp")
        model = self._model_struct(present)
        stream = torch.cuda.current_stream(dev).cuda_stream
        if num_neigh is None:
            check(lib.matpl_dp_eval(self.code, ctypes.byref(model), B, N, S, nghost, ptr(ln),
                                    ptr(idr), ptr(tm), ptr(out["Ei_atom"]), ptr(out["Etot"]),
                                    ptr(out["Force"]), ptr(out["Virial"]), ptr(ws), ws.numel(),
                                    stream), "matpl_dp_eval")
        else:
            nn = num_neigh if num_neigh.dtype == torch.int32 and num_neigh.is_contiguous() \
                else num_neigh.to(torch.int32).contiguous()
            if nn.numel() != B * N * self.cfg.ntypes:
                raise _lib.MatplError("num_neigh must be [B, N, ntypes]")
            check(lib.matpl_dp_eval_occupied(self.code, ctypes.byref(model), B, N, S, nghost,
                                             ptr(ln), ptr(nn), ptr(idr), ptr(tm),
                                             ptr(out["Ei_atom"]), ptr(out["Etot"]),
                                             ptr(out["Force"]), ptr(out["Virial"]), ptr(ws),
                                             ws.numel(), stream), "matpl_dp_eval_occupied")
        if self.check_errors:
            code = int(self.err.item())
            if code:
                self.err.zero_()
                if code == _lib.KERR_TIMEOUT:
                    raise _lib.MatplError("matpl_dp_eval: a tensor-core completion wait gave up "
                                          "(MATPL_KERR_TIMEOUT); the outputs are invalid")
                raise _lib.MatplError(f"matpl_dp_eval kernel error code {code}")
        return out

    def forward(self, list_neigh, Imagetype_map, atom_type, ImageDR, nghost: int = 0,
                Egroup_weight=None, divider=None, is_calc_f: Optional[bool] = True):
        present = self.present_types(atom_type)
        tm = Imagetype_map.to(device=ImageDR.device, dtype=torch.int32)
        r = self.evaluate(list_neigh, tm, present, ImageDR, int(nghost))
        perm = self._grouped_perm(tm, present)
        Ei = r["Ei_atom"][:, perm]
        Etot = r["Etot"].to(self.dtype).unsqueeze(-1)
        Egroup = None
        if Egroup_weight is not None and divider is not None:   # dp_dp.py:105-124
            Egroup = torch.divide(torch.matmul(Egroup_weight, Ei.unsqueeze(-1)).squeeze(-1), divider)
        if is_calc_f is False:
            return Etot, Ei, None, Egroup, None
        return Etot, Ei, r["Force"], Egroup, r["Virial"].to(self.dtype)
