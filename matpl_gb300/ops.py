"""Drop-in replacements for MatPL's ``CalcOps_cuda`` DP ops and data-path builders.

``calculateForce`` / ``calculateVirial`` keep the reference signatures and return lists like
``torch.ops.CalcOps_cuda.*`` (src/op/src/CalcOps_bind.cpp:6-16, CalcOps.cpp:6-236) and are
differentiable w.r.t. ``dE`` exactly like the reference ``autograd::Function``s.  ``find_neighbore``
mirrors ``src/pre_data/dpuni_data_loader.py:595-650`` on the GPU and ``env_mat`` mirrors
``DP.calculate_Ri`` (``src/model/dp_dp.py:217-302``).

Every op runs on the current CUDA stream of its inputs' device, goes through the C ABI of
``libmatpl_gb300.so`` and raises ``MatplError`` on failure; there is no CPU fallback.
"""
from typing import List, Optional, Sequence, Tuple, Union

import torch

from . import _lib
from ._lib import MATPL_F32, MATPL_F64, check, ptr

_DT = {torch.float32: MATPL_F32, torch.float64: MATPL_F64}


def _stream(dev: torch.device) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


def _dtype_code(t: torch.Tensor) -> int:
    if t.dtype not in _DT:
        raise _lib.MatplError(f"unsupported dtype {t.dtype}; MatPL DP ops take float32/float64")
    return _DT[t.dtype]


def _require_cuda(*ts):
    for t in ts:
        if t is not None and not t.is_cuda:
            raise _lib.MatplError("matpl_gb300 ops take CUDA tensors (no CPU fallback)")


def _nghost(n) -> int:
    return int(n.item()) if isinstance(n, torch.Tensor) else int(n)


class _CalculateForce(torch.autograd.Function):
    @staticmethod
    @_lib.on_device
    def forward(ctx, list_neigh, dE, Ri_d, F, nghost: int):
        B, N = list_neigh.shape[0], list_neigh.shape[1]
        S = list_neigh[0, 0].numel() if N > 0 else 0
        nl = list_neigh.contiguous().to(torch.int32)
        dE_c, Rd = dE.contiguous(), Ri_d.contiguous()
        out = torch.empty(B, N + nghost, 3, dtype=dE.dtype, device=dE.device)
        lib = _lib.load()
        check(lib.matpl_calc_force(_dtype_code(dE), ptr(nl), ptr(dE_c), ptr(Rd),
                                   ptr(F.contiguous().to(dE.dtype)), B, N, S, nghost, ptr(out),
                                   _stream(dE.device)), "matpl_calc_force")
        ctx.save_for_backward(nl, Rd)
        ctx.meta = (B, N, S, nghost, dE.shape)
        return out

    @staticmethod
    @_lib.on_device
    def backward(ctx, grad_force):
        nl, Rd = ctx.saved_tensors
        B, N, S, nghost, dshape = ctx.meta
        g = grad_force.contiguous()
        grad = torch.empty(dshape, dtype=Rd.dtype, device=Rd.device)
        lib = _lib.load()
        check(lib.matpl_calc_force_grad(_dtype_code(Rd), ptr(nl), ptr(Rd), ptr(g), B, N, S,
                                        nghost, ptr(grad), _stream(Rd.device)),
              "matpl_calc_force_grad")
        return None, grad, None, None, None


class _CalculateVirial(torch.autograd.Function):
    @staticmethod
    @_lib.on_device
    def forward(ctx, list_neigh, dE, Rij, Ri_d, nghost: int):
        B, N = list_neigh.shape[0], list_neigh.shape[1]
        S = list_neigh[0, 0].numel() if N > 0 else 0
        nl = list_neigh.contiguous().to(torch.int32)
        dE_c, Rj, Rd = dE.contiguous(), Rij.contiguous().to(dE.dtype), Ri_d.contiguous()
        vir = torch.empty(B, 9, dtype=dE.dtype, device=dE.device)
        avir = torch.empty(B, N + nghost, 9, dtype=dE.dtype, device=dE.device)
        lib = _lib.load()
        check(lib.matpl_calc_virial(_dtype_code(dE), ptr(nl), ptr(dE_c), ptr(Rj), ptr(Rd), B, N,
                                    S, nghost, ptr(vir), ptr(avir), _stream(dE.device)),
              "matpl_calc_virial")
        ctx.save_for_backward(nl, Rj, Rd)
        ctx.meta = (B, N, S, dE.shape)
        ctx.mark_non_differentiable(avir)
        return vir, avir

    @staticmethod
    @_lib.on_device
    def backward(ctx, grad_vir, grad_avir):
        nl, Rj, Rd = ctx.saved_tensors
        B, N, S, dshape = ctx.meta
        grad = torch.empty(dshape, dtype=Rd.dtype, device=Rd.device)
        g = grad_vir.contiguous() if grad_vir is not None else torch.zeros(
            B, 9, dtype=Rd.dtype, device=Rd.device)
        lib = _lib.load()
        check(lib.matpl_calc_virial_grad(_dtype_code(Rd), ptr(nl), ptr(Rj), ptr(Rd), ptr(g), B, N,
                                         S, ptr(grad), _stream(Rd.device)),
              "matpl_calc_virial_grad")
        return None, grad, None, None, None


def calculateForce(list_neigh: torch.Tensor, dE: torch.Tensor, Ri_d: torch.Tensor,
                   F: torch.Tensor, nghost_tensor) -> List[torch.Tensor]:
    """``CalcOps_cuda.calculateForce`` (CalcOps.cpp:6-72).

    list_neigh [B,N,1,S] int32 0-based (-1 empty), dE [B,N,1,4S], Ri_d [B,N,4S,3],
    F [B,N,3] (centre term), nghost 0-d int64 tensor or int -> [force [B,N+nghost,3]]."""
    _require_cuda(list_neigh, dE, Ri_d, F)
    return [_CalculateForce.apply(list_neigh, dE, Ri_d, F, _nghost(nghost_tensor))]


def calculateVirial(list_neigh: torch.Tensor, dE: torch.Tensor, Rij: torch.Tensor,
                    Ri_d: torch.Tensor, nghost_tensor) -> List[torch.Tensor]:
    """``CalcOps_cuda.calculateVirial`` (CalcOps.cpp:170-236) -> [virial [B,9],
    atom_virial [B,N+nghost,9]], virial[a*3+c] = sum f_a Rij_c."""
    _require_cuda(list_neigh, dE, Rij, Ri_d)
    v, av = _CalculateVirial.apply(list_neigh, dE, Rij, Ri_d, _nghost(nghost_tensor))
    return [v, av]


class _CalculateCompress(torch.autograd.Function):
    @staticmethod
    @_lib.on_device
    def forward(ctx, f2, coefficient):
        ns, nodes, nc = coefficient.shape
        f = f2.contiguous().reshape(-1).to(coefficient.dtype)
        c = coefficient.contiguous()
        G = torch.empty(ns, nodes, dtype=c.dtype, device=c.device)
        check(_lib.load().matpl_calc_compress(_dtype_code(c), ptr(f), ptr(c), ns, nodes, nc, ptr(G),
                                              _stream(c.device)), "matpl_calc_compress")
        ctx.save_for_backward(f, c)
        ctx.f2_shape = f2.shape
        return G

    @staticmethod
    @_lib.on_device
    def backward(ctx, grad_G):
        f, c = ctx.saved_tensors
        ns, nodes, nc = c.shape
        g = grad_G.contiguous().to(c.dtype)
        out = torch.empty(ns, dtype=c.dtype, device=c.device)
        check(_lib.load().matpl_calc_compress_grad(_dtype_code(c), ptr(f), ptr(c), ptr(g), ns, nodes,
                                                   nc, ptr(out), _stream(c.device)),
              "matpl_calc_compress_grad")
        return out.reshape(ctx.f2_shape), None


def calculateCompress(f2: torch.Tensor, coefficient: torch.Tensor) -> List[torch.Tensor]:
    """``CalcOps_cuda.calculateCompress`` (CalcOps.cpp:331-383): f2 [nsij,1], coefficient
    [nsij, layer_node, 4 or 6] (highest power first) -> [G [nsij, layer_node]]; differentiable
    in f2 like the reference (no gradient for the coefficients)."""
    _require_cuda(f2, coefficient)
    return [_CalculateCompress.apply(f2, coefficient)]


@_lib.on_device
def env_mat(ImageDR: torch.Tensor, Imagetype_map: torch.Tensor, davg: torch.Tensor,
            dstd: torch.Tensor, Rmin: float, Rmax: float) -> Tuple[torch.Tensor, torch.Tensor]:
    """``DP.calculate_Ri`` (dp_dp.py:217-302): normalised Ri [B,N,S,4] and Ri_d [B,N,S,4,3]."""
    _require_cuda(ImageDR, Imagetype_map)
    B, N, S, _ = ImageDR.shape
    dt = ImageDR.dtype
    idr = ImageDR.contiguous()
    tm = Imagetype_map.to(device=ImageDR.device, dtype=torch.int32).contiguous()
    av = davg.to(device=ImageDR.device, dtype=dt).contiguous()
    sd = dstd.to(device=ImageDR.device, dtype=dt).contiguous()
    Ri = torch.empty(B, N, S, 4, dtype=dt, device=ImageDR.device)
    Rid = torch.empty(B, N, S, 4, 3, dtype=dt, device=ImageDR.device)
    lib = _lib.load()
    check(lib.matpl_env_mat(_dtype_code(ImageDR), B, N, S, ptr(tm), ptr(idr), ptr(av), ptr(sd),
                            float(Rmin), float(Rmax), ptr(Ri), ptr(Rid), _stream(ImageDR.device)),
          "matpl_env_mat")
    return Ri, Rid


class NeighborOverflow(_lib.MatplError):
    """A type block needs more than maxNeighborNum slots (NeighConst.f90:75-78)."""


_ws_cache = {}


def workspace(device: torch.device, nbytes: int, tag: str) -> torch.Tensor:
    """Grow-only scratch buffer per (device, current stream, tag); the C ABI itself never
    allocates.  Keying by the stream keeps calls on different streams from sharing one buffer
    (they could overlap on the GPU), and a buffer that is replaced by a larger one was only
    ever used on that stream, so the allocator may hand it out again in stream order."""
    device = torch.device(device)
    stream = torch.cuda.current_stream(device).cuda_stream
    key = (str(device), stream, tag)
    buf = _ws_cache.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=device)
        _ws_cache[key] = buf
    return buf


@_lib.on_device
def find_neighbore(type_maps: torch.Tensor, frac_position: torch.Tensor, lattice: torch.Tensor,
                   ntypes: int, m_neigh: int, Rc_M: float, Rc_type: Union[float, Sequence[float]],
                   out_dtype: torch.dtype = torch.float64, with_counts: bool = False,
                   check_overflow: bool = True, occupied_only: bool = False):
    """GPU DP neighbor search (dpuni_data_loader.py:595-650 + compute_Ri's r column).

    type_maps [N] 0-based types; frac_position [B,N,3] (or [N,3]) f64 fractional; lattice
    [B,3,3] (or [3,3]) f64 row vectors.  Returns list_neigh [B,N,ntypes*m] int32 (1-based,
    0 = empty) and ImageDR [B,N,ntypes*m,4] = (r, dx, dy, dz) (plus num_neigh [B,N,ntypes]
    when ``with_counts``).  Raises NeighborOverflow like the Fortran "stop" when
    ``check_overflow`` (that reads one device flag and synchronises the stream).
    ``occupied_only`` writes only the occupied slots (the empty ones hold whatever the
    fresh tensors held) and always returns the counts; pass them to ``DP.evaluate``."""
    _require_cuda(frac_position)
    dev = frac_position.device
    pos = frac_position.to(torch.float64)
    N = type_maps.shape[0]
    pos = pos.reshape(-1, N, 3).contiguous()
    B = pos.shape[0]
    lat = lattice.to(device=dev, dtype=torch.float64).reshape(B, 3, 3).contiguous()
    tm = type_maps.to(device=dev, dtype=torch.int32).contiguous()
    rct = [float(Rc_type)] * ntypes if isinstance(Rc_type, (int, float)) else [float(x) for x in Rc_type]
    if len(rct) != ntypes:
        raise _lib.MatplError("Rc_type must have ntypes entries")
    import ctypes
    rct_c = (ctypes.c_double * ntypes)(*rct)
    S = ntypes * m_neigh
    ln = torch.empty(B, N, S, dtype=torch.int32, device=dev)
    idr = torch.empty(B, N, S, 4, dtype=out_dtype, device=dev)
    with_counts = with_counts or occupied_only
    cnt = torch.empty(B, N, ntypes, dtype=torch.int32, device=dev) if with_counts else None
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    lib = _lib.load()
    nbytes = lib.matpl_neighbor_workspace_bytes(B, N)
    ws = workspace(dev, nbytes, "neighbor")
    build = lib.matpl_neighbor_build_occupied if occupied_only else lib.matpl_neighbor_build
    check(build(B, N, ntypes, m_neigh, float(Rc_M), rct_c, ptr(tm), ptr(lat), ptr(pos),
                _DT[out_dtype], ptr(ln), ptr(idr), ptr(cnt), ptr(err), ptr(ws), ws.numel(),
                _stream(dev)), "matpl_neighbor_build")
    if check_overflow:
        code = int(err.item())
        if code == _lib.KERR_NEIGHBOR_OVERFLOW:
            raise NeighborOverflow(f"Error! maxNeighborNum too small {m_neigh}")
        if code == _lib.KERR_BAD_BOX:
            raise _lib.MatplError("matpl_neighbor_build: the cell is so small that natoms x "
                                  "periodic images exceeds 2^31")
        if code != 0:
            raise _lib.MatplError(f"matpl_neighbor_build kernel error {code} (bad atom type)")
    if with_counts:
        return ln, idr, cnt
    return ln, idr


# ----------------------------------------------------------------------------------------------
# NEP neighbor operators (CalcOps.calculate_neighbor / calculate_maxneigh, CalcOps.cpp:1025-1172)
# ----------------------------------------------------------------------------------------------
def _nep_frames(num_atoms, box, box_orig, num_cell, position):
    _require_cuda(position)
    dev = position.device
    na = num_atoms.to(device=dev, dtype=torch.int64).reshape(-1).contiguous()
    B = na.shape[0]
    bx = box.to(device=dev, dtype=torch.float64).reshape(B, 18).contiguous()
    bo = box_orig.to(device=dev, dtype=torch.float64).reshape(B, 9).contiguous()
    nc = num_cell.to(device=dev, dtype=torch.int64).reshape(B, 3).contiguous()
    pos = position.to(torch.float64).reshape(-1, 3).contiguous()
    return dev, na, bx, bo, nc, pos


def _nep_kernel_error(err: torch.Tensor, what: str):
    code = int(err.item())
    if code == _lib.KERR_NEIGHBOR_OVERFLOW:
        raise NeighborOverflow(f"{what}: a neighbor list is longer than max_NN")
    if code:
        raise _lib.MatplError(f"{what} kernel error code {code}")


@_lib.on_device
def calculate_maxneigh(num_atoms: torch.Tensor, box: torch.Tensor, box_orig: torch.Tensor,
                       num_cell: torch.Tensor, position: torch.Tensor, cutoff_2b: float,
                       cutoff_3b: float, atom_type_num: int, atom_type_map: torch.Tensor,
                       with_type: bool) -> List[torch.Tensor]:
    """Neighbor counts [NN_radial, NN_angular], each [N] (or [N * ntypes] per neighbor element
    when ``with_type``), as ``CalcOps.calculate_maxneigh`` returns them."""
    dev, na, bx, bo, nc, pos = _nep_frames(num_atoms, box, box_orig, num_cell, position)
    N = pos.shape[0]
    nt = int(atom_type_num) if with_type else 1
    tm = atom_type_map.to(device=dev, dtype=torch.int64).contiguous()
    NN_r = torch.empty(N * nt, dtype=torch.int64, device=dev)
    NN_a = torch.empty(N * nt, dtype=torch.int64, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    lib = _lib.load()
    ws = workspace(dev, lib.matpl_nep_neighbor_workspace_bytes(na.shape[0], N), "nep_neighbor")
    check(lib.matpl_nep_maxneigh(na.shape[0], N, ptr(na), ptr(bx), ptr(bo), ptr(nc), ptr(pos),
                                 float(cutoff_2b), float(cutoff_3b), int(atom_type_num), ptr(tm),
                                 int(bool(with_type)), ptr(NN_r), ptr(NN_a), ptr(err), ptr(ws),
                                 ws.numel(), _stream(dev)), "matpl_nep_maxneigh")
    _nep_kernel_error(err, "calculate_maxneigh")
    return [NN_r, NN_a]


@_lib.on_device
def calculate_neighbor(num_atoms: torch.Tensor, atom_type_map: torch.Tensor,
                       atom_types: torch.Tensor, box: torch.Tensor, box_orig: torch.Tensor,
                       num_cell: torch.Tensor, position: torch.Tensor, cutoff_2b: float,
                       cutoff_3b: float, max_NN_radial: int, max_NN_angular: int,
                       with_rij: bool, check_overflow: bool = True) -> List[torch.Tensor]:
    """[NN_radial, NN_angular, NL_radial, NL_angular, Ri_radial, Ri_angular] exactly as
    ``CalcOps.calculate_neighbor`` returns them (atom_type_map / atom_types are accepted for
    signature compatibility; the lists do not depend on them).  A list longer than max_NN
    raises NeighborOverflow when ``check_overflow`` (one device read)."""
    dev, na, bx, bo, nc, pos = _nep_frames(num_atoms, box, box_orig, num_cell, position)
    N = pos.shape[0]
    w = 4 if with_rij else 3
    mr, ma = int(max_NN_radial), int(max_NN_angular)
    NN_r = torch.empty(N, dtype=torch.int64, device=dev)
    NN_a = torch.empty(N, dtype=torch.int64, device=dev)
    NL_r = torch.empty(N, mr, dtype=torch.int64, device=dev)
    NL_a = torch.empty(N, ma, dtype=torch.int64, device=dev)
    Ri_r = torch.empty(N, mr, w, dtype=torch.float64, device=dev)
    Ri_a = torch.empty(N, ma, w, dtype=torch.float64, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    lib = _lib.load()
    ws = workspace(dev, lib.matpl_nep_neighbor_workspace_bytes(na.shape[0], N), "nep_neighbor")
    check(lib.matpl_nep_neighbor(na.shape[0], N, ptr(na), ptr(bx), ptr(bo), ptr(nc), ptr(pos),
                                 float(cutoff_2b), float(cutoff_3b), mr, ma, int(bool(with_rij)),
                                 ptr(NN_r), ptr(NN_a), ptr(NL_r), ptr(NL_a), ptr(Ri_r), ptr(Ri_a),
                                 ptr(err), ptr(ws), ws.numel(), _stream(dev)),
          "matpl_nep_neighbor")
    if check_overflow:
        _nep_kernel_error(err, "calculate_neighbor")
    return [NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a]


class SkinNeighbor:
    """Verlet-skin reuse of ``calculate_neighbor``'s lists for a caller that steps one fixed box
    (molecular dynamics).  ``lists(position)`` returns what ``calculate_neighbor`` returns at
    that position, bit for bit (same pairs, same order, same values), but rebuilds its skin list
    (all pairs within max cutoff + ``skin``) only when some atom has moved more than skin / 2
    since the last build, the rule of ``pair_matpl.cpp:1096-1110``; otherwise it filters the
    skin list with the search's own FP64 arithmetic.  The rebuild decision is taken on the
    device, so the call (and an evaluation after it) can be captured in a CUDA graph.

    ``compact=True`` is the MD form: the lists are int32 NN / NL and f32 Ri [N, max_NN, 4]
    = (r, x, y, z), made in FP32 from each pair's vector at the build plus the two atoms'
    displacements since then (a few FP32 ulps from the exact vectors; entries past NN are not
    written); ``nep.NEP.evaluate`` takes them in float32.

    The returned tensors are owned by this object and overwritten by the next call.  The box is
    fixed: ``set_box`` replaces it and forces a rebuild.  Every frame must be a single cell at
    least three (max cutoff + skin)-wide cells thick; other boxes raise ValueError (use
    ``calculate_neighbor``).  ``capacity`` (skin-list slots per atom) defaults to 1.25 x the
    largest count within max cutoff + skin at the first positions, plus 16."""

    def __init__(self, num_atoms: torch.Tensor, box: torch.Tensor, box_orig: torch.Tensor,
                 num_cell: torch.Tensor, position: torch.Tensor, cutoff_2b: float,
                 cutoff_3b: float, max_NN_radial: int, max_NN_angular: int,
                 with_rij: bool = True, skin: float = 1.0, capacity: Optional[int] = None,
                 compact: bool = False):
        dev, na, bx, bo, nc, pos = _nep_frames(num_atoms, box, box_orig, num_cell, position)
        if skin < 0:
            raise ValueError("skin must be >= 0")
        if compact and not with_rij:
            raise ValueError("the compact lists always carry r (with_rij)")
        self.compact = bool(compact)
        self.device = dev
        self.na, self.bx, self.bo, self.nc = na, bx, bo, nc
        self.N = pos.shape[0]
        self.rc = (float(cutoff_2b), float(cutoff_3b))
        self.skin = float(skin)
        # a hair above max(rc) + skin: a pair just inside rc after moves just under skin / 2
        # each stays inside r_list whatever the last-bit rounding of the two distances
        self.r_list = max(self.rc) + self.skin + 1e-6
        self.mr, self.ma = int(max_NN_radial), int(max_NN_angular)
        self.width = 4 if with_rij else 3
        if capacity is None:
            zeros = torch.zeros(self.N, dtype=torch.int64, device=dev)
            cnt, _ = calculate_maxneigh(na, bx, bo, nc, pos, self.r_list, min(self.rc), 1,
                                        zeros, False)
            capacity = int(int(cnt.max()) * 1.25) + 16 if self.N else 16
        self.cap = int(capacity)
        i32 = dict(dtype=torch.int32, device=dev)
        self.skin_nbr = torch.empty(self.N, self.cap, **i32)
        self.skin_cnt = torch.zeros(self.N, **i32)
        self.x_ref = torch.zeros(self.N, 3, dtype=torch.float64, device=dev)
        self.skin_vec = (torch.zeros(self.N, self.cap, 4, dtype=torch.float32, device=dev)
                         if compact else None)
        self.delta = torch.zeros(self.N, 4, dtype=torch.float32, device=dev) if compact else None
        self.gate = torch.ones(1, **i32)
        self.nbuild = torch.zeros(1, **i32)
        self.err = torch.zeros(1, **i32)
        lib = _lib.load()
        self.ws = torch.empty(max(256, lib.matpl_nep_neighbor_workspace_bytes(na.shape[0],
                                                                              self.N)),
                              dtype=torch.uint8, device=dev)
        N, w = self.N, self.width
        it, ft = (torch.int32, torch.float32) if compact else (torch.int64, torch.float64)
        self.out = [torch.empty(N, dtype=it, device=dev),
                    torch.empty(N, dtype=it, device=dev),
                    torch.empty(N, self.mr, dtype=it, device=dev),
                    torch.empty(N, self.ma, dtype=it, device=dev),
                    torch.empty(N, self.mr, w, dtype=ft, device=dev),
                    torch.empty(N, self.ma, w, dtype=ft, device=dev)]
        if compact:      # entries past NN are never written: keep them defined
            for t, v in zip(self.out[2:], (-1, -1, 0, 0)):
                t.fill_(v)
        self.lists(pos)
        code = int(self.err.item())
        if code == _lib.KERR_BAD_BOX:
            raise ValueError("SkinNeighbor: a frame is not one cell at least three "
                             f"{self.r_list:.3f} A cells thick; use calculate_neighbor")
        self.check_errors()

    @_lib.on_device
    def lists(self, position: torch.Tensor) -> List[torch.Tensor]:
        """[NN_radial, NN_angular, NL_radial, NL_angular, Ri_radial, Ri_angular] at
        ``position`` ([N, 3] f64 cartesian, on this object's device)."""
        pos = position
        if not (pos.dtype == torch.float64 and pos.is_contiguous()):
            pos = pos.to(torch.float64).contiguous()
        if pos.device != self.device or pos.numel() != 3 * self.N:
            raise _lib.MatplError(f"SkinNeighbor: position must be [{self.N}, 3] on {self.device}")
        lib = _lib.load()
        s = _stream(self.device)
        B = self.na.shape[0]
        check(lib.matpl_nep_skin_update(B, self.N, ptr(self.na), ptr(self.bx), ptr(self.bo),
                                        ptr(self.nc), ptr(pos), self.r_list, self.skin, self.cap,
                                        ptr(self.skin_nbr), ptr(self.skin_cnt), ptr(self.x_ref),
                                        ptr(self.skin_vec), ptr(self.delta), ptr(self.gate),
                                        ptr(self.nbuild), ptr(self.err), ptr(self.ws),
                                        self.ws.numel(), s),
              "matpl_nep_skin_update")
        o = self.out
        if self.compact:
            check(lib.matpl_nep_skin_filter_compact(
                self.N, self.rc[0], self.rc[1], self.mr, self.ma, self.cap, ptr(self.skin_nbr),
                ptr(self.skin_cnt), ptr(self.skin_vec), ptr(self.delta), ptr(o[0]), ptr(o[1]),
                ptr(o[2]), ptr(o[3]), ptr(o[4]), ptr(o[5]), ptr(self.err), s),
                "matpl_nep_skin_filter_compact")
            return o
        check(lib.matpl_nep_skin_filter(B, self.N, ptr(pos), self.rc[0], self.rc[1], self.mr,
                                        self.ma, int(self.width == 4), self.cap,
                                        ptr(self.skin_nbr), ptr(self.skin_cnt), ptr(o[0]),
                                        ptr(o[1]), ptr(o[2]), ptr(o[3]), ptr(o[4]), ptr(o[5]),
                                        ptr(self.err), ptr(self.ws), self.ws.numel(), s),
              "matpl_nep_skin_filter")
        return o

    __call__ = lists

    def set_box(self, box: torch.Tensor, box_orig: torch.Tensor, num_cell: torch.Tensor):
        """Replace the box (same frames and atoms); the next call rebuilds."""
        B = self.na.shape[0]
        self.bx.copy_(box.reshape(B, 18))
        self.bo.copy_(box_orig.reshape(B, 9))
        self.nc.copy_(num_cell.reshape(B, 3))
        self.force_rebuild()

    def force_rebuild(self):
        self.gate.fill_(1)

    def rebuilds(self) -> int:
        """Skin-list builds so far (one device read)."""
        return int(self.nbuild.item())

    def check_errors(self):
        """Raise on a kernel error recorded since the last check (one device read): a list
        longer than max_NN or a skin list longer than its capacity raises NeighborOverflow."""
        code = int(self.err.item())
        if code:
            self.err.zero_()
            if code == _lib.KERR_NEIGHBOR_OVERFLOW:
                raise NeighborOverflow("SkinNeighbor: a list is longer than max_NN or the skin "
                                       f"capacity {self.cap}")
            raise _lib.MatplError(f"SkinNeighbor kernel error code {code}")


# NEP training operators (CalcOps.calculateNepFeat / calculateNepMbFeat / calculateNepForce /
# calculateNepVirial) live in nep_ops (which builds on this module) and resolve here on access
_NEP_OPS = ("calculateNepFeat", "calculateNepMbFeat", "calculateNepForce", "calculateNepVirial")


def __getattr__(name):
    if name in _NEP_OPS:
        from . import nep_ops
        return getattr(nep_ops, name)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")

