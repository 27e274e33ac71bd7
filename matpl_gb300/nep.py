"""NEP model description on the host: hyper-parameters, parameters, periodic box expansion.

Mirrors the parts of MatPL that the NEP evaluation path reads:

* ``NepConfig``: ``NepParam`` (src/user/nep_param.py:51-83) - cutoff [radial, angular], n_max,
  basis_size, l_max [3-body, 4-body, 5-body], neuron [hidden, 1], train_2b, zbl - plus the
  element list (atomic numbers); ``feature_nums`` follows ``NEP.set_init_nep_param`` (src/model/nep_net.py:111-143).
* ``init_params``: seeded parameters of the shapes ``NEP`` holds - ``c_param_2``
  [T, T, n_max_r + 1, basis_r + 1], ``c_param_3`` [T, T, n_max_a + 1, basis_a + 1]
  (nep_net.py:160-176), one single-hidden-layer ``FittingNet`` per element
  (src/model/nep_fitting.py:40-95) and ``q_scaler`` [F].
* ``calc_q_scaler``: ``NEP.update_scaler_values`` (nep_net.py:1020-1058), q_scaler = 1/(max-min)
  with shared extrema over each (l, body-order) block.
* ``expand_box``: ``UniDataset.expand_box`` (src/pre_data/nep_data_loader.py:220-253): the number
  of replicas per lattice direction, the replicated cell h (columns = vectors) and h^-1.
* ``pack_params``: the flat device layout of ``matpl_nep_eval``.
"""
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import math

import numpy as np
import torch

from . import _lib


@dataclass
class NepConfig:
    atom_type: List[int]
    cutoff: Sequence[float] = (6.0, 4.0)
    n_max: Sequence[int] = (4, 4)
    basis_size: Sequence[int] = (8, 8)
    l_max: Sequence[int] = (4, 2, 1)
    neuron: int = 30
    train_2b: bool = True
    zbl: Optional[float] = None     # outer cutoff of the ZBL term (nep_param.zbl), None = off

    @property
    def ntypes(self) -> int:
        return len(self.atom_type)

    @property
    def nr(self) -> int:          # radial descriptor components n = 0..n_max_r
        return self.n_max[0] + 1

    @property
    def na(self) -> int:          # angular radial functions n = 0..n_max_a
        return self.n_max[1] + 1

    @property
    def kr(self) -> int:          # Chebyshev basis functions k = 0..basis_r
        return self.basis_size[0] + 1

    @property
    def ka(self) -> int:
        return self.basis_size[1] + 1

    @property
    def two_feat_num(self) -> int:
        return self.nr if self.train_2b else 0

    @property
    def multi_feat_num(self) -> int:
        l3, l4, l5 = self.l_max
        if l3 <= 0:
            return 0
        return self.na * l3 + (self.na if l4 > 0 else 0) + (self.na if l5 > 0 else 0)

    @property
    def feature_nums(self) -> int:
        return self.two_feat_num + self.multi_feat_num


def init_params(cfg: NepConfig, seed: int, energy_shift: float = 0.0,
                dtype=torch.float64) -> Dict[str, torch.Tensor]:
    """Seeded parameters with the reference's shapes and initial distributions: c = U(-0.5, 0.5)
    + 0.1 N(0, 1) (nep_net.py:166-170); hidden weight N(0, 1/sqrt(F + H)), bias N(0, 1); output
    weight N(0, 1/sqrt(H + 1)), bias N(energy_shift, 1) (nep_fitting.py:62-91).  q_scaler is set
    to 1; ``calc_q_scaler`` replaces it from descriptor statistics."""
    g = torch.Generator().manual_seed(seed)
    T, F, H = cfg.ntypes, cfg.feature_nums, cfg.neuron

    def cparam(n, k):
        m = torch.rand(T, T, n, k, generator=g, dtype=torch.float64) - 0.5
        return m + 0.1 * torch.randn(T, T, n, k, generator=g, dtype=torch.float64)

    p = {"c_param_2": cparam(cfg.nr, cfg.kr)}
    if cfg.l_max[0] > 0:
        p["c_param_3"] = cparam(cfg.na, cfg.ka)
    for t in range(T):
        pre = f"fitting_net.{t}.layers."
        p[pre + "0.weight"] = torch.randn(F, H, generator=g, dtype=torch.float64) / math.sqrt(F + H)
        p[pre + "0.bias"] = torch.randn(1, H, generator=g, dtype=torch.float64)
        p[pre + "1.weight"] = torch.randn(H, 1, generator=g, dtype=torch.float64) / math.sqrt(H + 1)
        p[pre + "1.bias"] = energy_shift + torch.randn(1, 1, generator=g, dtype=torch.float64)
    p["q_scaler"] = torch.ones(F, dtype=torch.float64)
    return {k: v.to(dtype) for k, v in p.items()}


def scaler_blocks(cfg: NepConfig):
    """Column ranges that share one extremum in ``update_scaler_values`` (nep_net.py:1027-1043):
    the radial block, one block per l of the 3-body part, the 4-body and the 5-body blocks."""
    blocks = [(0, cfg.two_feat_num)]
    off = cfg.two_feat_num
    l3, l4, l5 = cfg.l_max
    if l3 > 0:
        for _ in range(l3):
            blocks.append((off, off + cfg.na))
            off += cfg.na
        if l4 > 0:
            blocks.append((off, off + cfg.na))
            off += cfg.na
        if l5 > 0:
            blocks.append((off, off + cfg.na))
    return [b for b in blocks if b[1] > b[0]]


def calc_q_scaler(cfg: NepConfig, feats: torch.Tensor) -> torch.Tensor:
    """q_scaler = 1 / (q_max - q_min), extrema taken per block over all atoms."""
    f = feats.reshape(-1, feats.shape[-1])
    qmax = f.max(0).values.clone()
    qmin = f.min(0).values.clone()
    for a, b in scaler_blocks(cfg):
        qmax[a:b] = qmax[a:b].max()
        qmin[a:b] = qmin[a:b].min()
    return 1.0 / (qmax - qmin)


def _det3(m: np.ndarray) -> float:
    return float(np.linalg.det(m.reshape(3, 3)))


def expand_box(lattice: np.ndarray, cutoff_radial: float):
    """(box [18], box_orig [9], num_cell [3], volume) for one frame.

    ``lattice`` has the lattice vectors as rows.  box_orig = lattice^T flattened, box[0:9] the
    replicated cell h with columns num_cell[k] * vector k, box[9:18] = adj(h) / det(h)."""
    lat = np.asarray(lattice, dtype=np.float64).reshape(3, 3)
    lt = lat.T.flatten()
    a, b, c = lt[0::3], lt[1::3], lt[2::3]

    def area(u, v):
        s1 = u[1] * v[2] - u[2] * v[1]
        s2 = u[2] * v[0] - u[0] * v[2]
        s3 = u[0] * v[1] - u[1] * v[0]
        return math.sqrt(s1 * s1 + s2 * s2 + s3 * s3)

    det = _det3(lt)
    volume = abs(det)
    num_cell = np.array([int(math.ceil(2.0 * cutoff_radial / (volume / area(b, c)))),
                         int(math.ceil(2.0 * cutoff_radial / (volume / area(c, a)))),
                         int(math.ceil(2.0 * cutoff_radial / (volume / area(a, b))))],
                        dtype=np.int64)
    box = np.zeros(18, dtype=np.float64)
    box[0:9:3] = lt[0::3] * num_cell[0]
    box[1:9:3] = lt[1::3] * num_cell[1]
    box[2:9:3] = lt[2::3] * num_cell[2]
    box[9] = box[4] * box[8] - box[5] * box[7]
    box[10] = box[2] * box[7] - box[1] * box[8]
    box[11] = box[1] * box[5] - box[2] * box[4]
    box[12] = box[5] * box[6] - box[3] * box[8]
    box[13] = box[0] * box[8] - box[2] * box[6]
    box[14] = box[2] * box[3] - box[0] * box[5]
    box[15] = box[3] * box[7] - box[4] * box[6]
    box[16] = box[1] * box[6] - box[0] * box[7]
    box[17] = box[0] * box[4] - box[1] * box[3]
    det *= float(num_cell[0] * num_cell[1] * num_cell[2])
    box[9:18] /= det
    return box, lt.copy(), num_cell, volume


@dataclass
class NepFrames:
    """A batch of frames in the reference's concatenated-atoms layout (nep_data_loader.py:200-215
    with ``variable_length_collate_fn``): cartesian positions [sum N, 3], per-atom element index,
    per-frame atom counts, box [B, 18], box_orig [B, 9], num_cell [B, 3]."""
    position: np.ndarray
    type_map: np.ndarray
    num_atom: np.ndarray
    box: np.ndarray
    box_orig: np.ndarray
    num_cell: np.ndarray
    volume: np.ndarray = field(default=None)

    @property
    def natoms(self) -> int:
        return int(self.position.shape[0])

    @property
    def nframes(self) -> int:
        return int(self.num_atom.shape[0])


def frames_from_structures(structs, cutoff_radial: float) -> NepFrames:
    """Concatenate ``matpl_gb300.structures.Structure`` objects (row-vector lattices, fractional
    coordinates, element indices) into the reference's NEP batch layout."""
    pos, tm, na, bx, bo, nc, vol = [], [], [], [], [], [], []
    for st in structs:
        box, lt, ncell, v = expand_box(st.lattice, cutoff_radial)
        pos.append(st.frac @ st.lattice)
        tm.append(np.asarray(st.types, dtype=np.int64))
        na.append(st.natoms)
        bx.append(box); bo.append(lt); nc.append(ncell); vol.append(v)
    return NepFrames(np.concatenate(pos), np.concatenate(tm), np.array(na, dtype=np.int64),
                     np.stack(bx), np.stack(bo), np.stack(nc), np.array(vol))


# ----------------------------------------------------------------------------------------------
# flat parameter layout of matpl_nep_eval (one contiguous buffer of the compute dtype):
#   c2 [T, T, nr, kr] | c3 [T, T, na, ka] | q_scaler [F] |
#   per type t: W0 [F, H] | b0 [H] | W1 [H] | b1 [1]
# ----------------------------------------------------------------------------------------------
def param_count(cfg: NepConfig) -> int:
    T, F, H = cfg.ntypes, cfg.feature_nums, cfg.neuron
    n = T * T * cfg.nr * cfg.kr + (T * T * cfg.na * cfg.ka if cfg.l_max[0] > 0 else 0) + F
    return n + T * (F * H + 2 * H + 1)


def pack_params(cfg: NepConfig, p: Dict[str, torch.Tensor]) -> torch.Tensor:
    parts = [p["c_param_2"].reshape(-1)]
    if cfg.l_max[0] > 0:
        parts.append(p["c_param_3"].reshape(-1))
    parts.append(p["q_scaler"].reshape(-1))
    for t in range(cfg.ntypes):
        pre = f"fitting_net.{t}.layers."
        parts += [p[pre + "0.weight"].reshape(-1), p[pre + "0.bias"].reshape(-1),
                  p[pre + "1.weight"].reshape(-1), p[pre + "1.bias"].reshape(-1)]
    flat = torch.cat([x.detach().to(torch.float64).cpu() for x in parts])
    assert flat.numel() == param_count(cfg)
    return flat


_SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga "
            "Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr "
            "Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr "
            "Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr").split()


def gpumd_text(cfg: NepConfig, p: Dict[str, torch.Tensor],
               max_neighbors: Sequence[int] = (500, 300)) -> str:
    """The model as a ``nep5`` potential file for LAMMPS / GPUMD (``extract_model``,
    utils/nep_to_gpumd.py:61-150): header lines (``nep5`` or ``nep5_zbl`` + ``zbl rc/2 rc``,
    cutoff with the list capacities, n_max, basis_size, l_max, ``ANN H 0``), then per element
    W0^T, -b0, W1 and -b1, a common bias 0, ``c_param_2`` and ``c_param_3`` as [n, k, t1, t2],
    and q_scaler.  Values are written with 9 significant digits, which round-trips every FP32
    value the reader parses them into."""
    T, F, H = cfg.ntypes, cfg.feature_nums, cfg.neuron
    names = [_SYMBOLS[z - 1] for z in cfg.atom_type]
    head = f"nep5{'_zbl' if cfg.zbl is not None else ''}   {T} {' '.join(names)}\n"
    if cfg.zbl is not None:
        head += f"zbl   {cfg.zbl / 2} {cfg.zbl}\n"
    head += (f"cutoff {cfg.cutoff[0]} {cfg.cutoff[1]} {int(max_neighbors[0])} "
             f"{int(max_neighbors[1])}\n")
    head += f"n_max  {' '.join(map(str, cfg.n_max))}\n"
    head += f"basis_size {' '.join(map(str, cfg.basis_size))}\n"
    head += f"l_max  {' '.join(map(str, cfg.l_max))}\n"
    head += f"ANN    {H} 0\n"
    f64 = lambda k: p[k].detach().to(torch.float64).cpu()  # noqa: E731
    vals = []
    for t in range(T):
        pre = f"fitting_net.{t}.layers."
        vals.append(f64(pre + "0.weight").t().reshape(-1))
        vals.append(-f64(pre + "0.bias").reshape(-1))
        vals.append(f64(pre + "1.weight").reshape(-1))
        vals.append(-f64(pre + "1.bias").reshape(-1))
    vals.append(torch.zeros(1, dtype=torch.float64))
    vals.append(f64("c_param_2").permute(2, 3, 0, 1).reshape(-1))
    if cfg.l_max[0] > 0:
        vals.append(f64("c_param_3").permute(2, 3, 0, 1).reshape(-1))
    vals.append(f64("q_scaler").reshape(-1))
    flat = torch.cat(vals).numpy().astype(np.float32)
    assert flat.size == T * (F * H + 2 * H + 1) + 1 + T * T * (
        cfg.nr * cfg.kr + (cfg.na * cfg.ka if cfg.l_max[0] > 0 else 0)) + F
    return head + "\n".join("%.9g" % float(v) for v in flat) + "\n"


# ----------------------------------------------------------------------------------------------
# GPU evaluator (the NEP.forward drop-in)
# ----------------------------------------------------------------------------------------------
NEP_PRECISIONS = {"float64": (1, torch.float64), "float32": (0, torch.float32)}


class NEP(torch.nn.Module):
    """Inference NEP on GB300 through ``matpl_nep_eval`` (plus ``matpl_nep_zbl`` when the
    model has a ZBL cutoff).

    ``forward`` takes what ``src/model/nep_net.py:NEP.forward`` takes (the six tensors of
    ``calculate_neighbor`` with with_rij, num_atom, atom_type_map) and returns
    (Etot [B, 1], Ei [N], Force [N, 3], Egroup, Virial [B, 9]).  ``precision`` "float32" runs the
    fused kernel in FP32 (FP64 energy / virial sums), "float64" in FP64."""

    def __init__(self, cfg: NepConfig, params: Dict[str, torch.Tensor], precision: str = "float32",
                 device="cuda", check_errors: bool = True):
        super().__init__()
        from . import _lib
        if precision not in NEP_PRECISIONS:
            raise _lib.MatplError(f"unknown precision {precision!r}; one of {list(NEP_PRECISIONS)}")
        self.cfg = cfg
        self.precision = precision
        self.code, self.dtype = NEP_PRECISIONS[precision]
        self.check_errors = check_errors
        dev = torch.device(device)
        self.device = dev
        self.register_buffer("packed", pack_params(cfg, params).to(device=dev, dtype=self.dtype))
        self.register_buffer("err", torch.zeros(1, dtype=torch.int32, device=dev))
        self._model = self._model_struct()
        lib = _lib.load()
        n = lib.matpl_nep_param_count(self._model)
        if n != self.packed.numel():
            raise _lib.MatplError(f"packed parameters {self.packed.numel()} != {n} expected")

    def _model_struct(self):
        from ._lib import MatplNepModel, ptr
        m = MatplNepModel()
        c = self.cfg
        m.ntypes = c.ntypes
        m.n_max_radial, m.basis_radial = c.n_max[0], c.basis_size[0]
        m.n_max_angular, m.basis_angular = c.n_max[1], c.basis_size[1]
        m.l_max_3b, m.l_max_4b, m.l_max_5b = c.l_max
        m.neuron = c.neuron
        m.train_2b = int(c.train_2b)
        m.cutoff_radial, m.cutoff_angular = float(c.cutoff[0]), float(c.cutoff[1])
        m.params = ptr(self.packed)
        m.err_dev = ptr(self.err)
        return m

    @_lib.on_device
    def evaluate(self, NN_radial, NL_radial, Ri_radial, NN_angular, NL_angular, Ri_angular,
                 num_atom, atom_type_map, out=None, descriptor_only: bool = False):
        """Raw evaluation: dict(Ei [N], Etot [B] f64, Force [N, 3], Virial [B, 9] f64).

        Takes calculate_neighbor's lists (int64 NN / NL, f64 Ri), or the compact MD lists of
        ``ops.SkinNeighbor(compact=True)`` (int32 NN / NL, f32 Ri; float32 models only)."""
        import ctypes
        from . import _lib
        from ._lib import check, ptr
        from .ops import workspace
        if not Ri_radial.is_cuda:
            raise _lib.MatplError("NEP.evaluate takes CUDA tensors (no CPU fallback)")
        dev = Ri_radial.device
        N = NL_radial.shape[0]
        na = num_atom.to(device=dev, dtype=torch.int64).reshape(-1).contiguous()
        B = na.shape[0]

        def i64(t):
            return t if (t.dtype == torch.int64 and t.is_contiguous()) else t.to(torch.int64).contiguous()

        def f64(t):
            return t if (t.dtype == torch.float64 and t.is_contiguous()) else t.to(torch.float64).contiguous()
        tm = i64(atom_type_map.to(dev))
        if Ri_radial.shape[-1] != 4 or Ri_angular.shape[-1] != 4:
            raise _lib.MatplError("Ri_radial / Ri_angular must be (r, x, y, z) (with_rij = True)")
        lib = _lib.load()
        ws = workspace(dev, lib.matpl_nep_workspace_bytes(self.code, B, N), "nep")
        stream = torch.cuda.current_stream(dev).cuda_stream
        if Ri_radial.dtype == torch.float32 and NL_radial.dtype == torch.int32:
            return self._evaluate_compact(NN_radial, NL_radial, Ri_radial, NN_angular, NL_angular,
                                          Ri_angular, na, tm, ws, stream, out, descriptor_only)
        lists = (NL_radial.shape[1], ptr(i64(NN_radial)), ptr(i64(NL_radial)), ptr(f64(Ri_radial)),
                 NL_angular.shape[1], ptr(i64(NN_angular)), ptr(i64(NL_angular)),
                 ptr(f64(Ri_angular)))
        if descriptor_only:
            feats = torch.empty(N, self.cfg.feature_nums, dtype=self.dtype, device=dev)
            check(lib.matpl_nep_descriptor(self.code, ctypes.byref(self._model), B, N, ptr(na),
                                           ptr(tm), *lists, ptr(feats), ptr(ws), ws.numel(),
                                           stream), "matpl_nep_descriptor")
            out = feats
        else:
            if out is None:
                out = {"Ei": torch.empty(N, dtype=self.dtype, device=dev),
                       "Etot": torch.empty(B, dtype=torch.float64, device=dev),
                       "Force": torch.empty(N, 3, dtype=self.dtype, device=dev),
                       "Virial": torch.empty(B, 9, dtype=torch.float64, device=dev)}
            check(lib.matpl_nep_eval(self.code, ctypes.byref(self._model), B, N, ptr(na), ptr(tm),
                                     *lists, ptr(out["Ei"]), ptr(out["Etot"]), ptr(out["Force"]),
                                     ptr(out["Virial"]), ptr(ws), ws.numel(), stream),
                  "matpl_nep_eval")
            if self.cfg.zbl is not None:                 # nep_net.py:399-408
                from . import nep_ops
                counts = tuple(int(c) for c in num_atom.reshape(-1).tolist())
                nep_ops.nep_zbl(self.cfg.zbl, self.cfg.atom_type, i64(NL_angular),
                                f64(Ri_angular), tm, counts, out["Ei"], out["Etot"], out["Force"],
                                out["Virial"])
        if self.check_errors:
            code = int(self.err.item())
            if code:
                self.err.zero_()
                raise _lib.MatplError(f"matpl_nep_eval kernel error code {code}")
        return out

    def _evaluate_compact(self, NN_r, NL_r, Ri_r, NN_a, NL_a, Ri_a, na, tm, ws, stream, out,
                          descriptor_only):
        import ctypes
        from . import _lib
        from ._lib import check, ptr
        if self.precision != "float32" or descriptor_only or self.cfg.zbl is not None:
            raise _lib.MatplError("the compact (int32 / f32) lists are evaluated by float32 "
                                  "models without ZBL, energy / force / virial only")
        ts = (NN_r, NL_r, Ri_r, NN_a, NL_a, Ri_a)
        if any(not t.is_contiguous() for t in ts) or NN_r.dtype != torch.int32 or \
                NN_a.dtype != torch.int32 or NL_a.dtype != torch.int32 or \
                Ri_a.dtype != torch.float32:
            raise _lib.MatplError("compact lists: contiguous int32 NN / NL and float32 Ri")
        N, B = NL_r.shape[0], na.shape[0]
        dev = Ri_r.device
        if out is None:
            out = {"Ei": torch.empty(N, dtype=torch.float32, device=dev),
                   "Etot": torch.empty(B, dtype=torch.float64, device=dev),
                   "Force": torch.empty(N, 3, dtype=torch.float32, device=dev),
                   "Virial": torch.empty(B, 9, dtype=torch.float64, device=dev)}
        lib = _lib.load()
        check(lib.matpl_nep_eval_compact(self.code, ctypes.byref(self._model), B, N, ptr(na),
                                         ptr(tm), NL_r.shape[1], ptr(NN_r), ptr(NL_r), ptr(Ri_r),
                                         NL_a.shape[1], ptr(NN_a), ptr(NL_a), ptr(Ri_a),
                                         ptr(out["Ei"]), ptr(out["Etot"]), ptr(out["Force"]),
                                         ptr(out["Virial"]), ptr(ws), ws.numel(), stream),
              "matpl_nep_eval_compact")
        if self.check_errors:
            code = int(self.err.item())
            if code:
                self.err.zero_()
                raise _lib.MatplError(f"matpl_nep_eval kernel error code {code}")
        return out

    def descriptor(self, NN_radial, NL_radial, Ri_radial, NN_angular, NL_angular, Ri_angular,
                   num_atom, atom_type_map):
        """feats [N, F] before q_scaler (the q of NEP.calculate_qn), compute dtype."""
        return self.evaluate(NN_radial, NL_radial, Ri_radial, NN_angular, NL_angular, Ri_angular,
                             num_atom, atom_type_map, descriptor_only=True)

    def forward(self, NN_radial, NL_radial, Ri_radial, NN_angular, NL_angular, Ri_angular,
                num_atom, atom_type_map, Egroup_weight=None, divider=None, is_calc_f=True):
        r = self.evaluate(NN_radial, NL_radial, Ri_radial, NN_angular, NL_angular, Ri_angular,
                          num_atom, atom_type_map)
        Ei = r["Ei"]
        Egroup = None
        if Egroup_weight is not None and divider is not None:      # nep_net.py:246-266
            Egroup = torch.divide(torch.matmul(Egroup_weight, Ei).squeeze(-1), divider)
        Etot = r["Etot"].to(self.dtype).unsqueeze(-1)
        if is_calc_f is False:
            return Etot, Ei, None, Egroup, None
        return Etot, Ei, r["Force"], Egroup, r["Virial"].to(self.dtype)
