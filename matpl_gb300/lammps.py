"""LAMMPS ``pair_style matpl`` for DP models, on the GB300.

Host-side mirror of the DP branch of ``PairMATPL`` (``src/lmps/lammps-libtorch/MATPL/
pair_matpl.cpp``): ``coeff`` maps LAMMPS types to model types (``:261-300``), ``compute``
(``:864-996``) turns LAMMPS' full neighbor list over local and ghost atoms into forces on
local and ghost atoms, the energy, the Voigt virial and per-atom energies.  The reference does
the list conversion on the host every step (``generate_neighdata``, ``:522-616``), copies the
expanded slot arrays (about 36 bytes per slot in FP64, ntypes * maxNeighborNum slots per atom)
to the GPU and runs the TorchScript model; here the raw list (4 bytes per entry) and the
positions go to the GPU and ``matpl_lammps_dp_compute`` builds the slots there
(``matpl_lammps_dp_neighbors``) and runs the fused evaluation with ghost rows.

``lammps_system`` is a stand-in for LAMMPS' own data in tests and benchmarks: periodic images
within the ghost cutoff as ghost atoms and a full list in random order, the layout a LAMMPS
``neighbor ... bin`` build hands a full-list pair style.
"""
import ctypes
from typing import Dict, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr
from .dp import DP

MIN_RSQ = 0.61   # pair_matpl.cpp:608: "there are two atoms too close" below this rsq


def _np(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class PairMATPL:
    """``pair_style matpl model.pt`` + ``pair_coeff * * <Z of each LAMMPS type>`` for one DP
    model.  ``eatom_grouped`` keeps the per-atom energies in the TorchScript model's order
    (grouped by LAMMPS type, what the reference stores in ``eatom``); False gives list-row
    order.  ``host_access``: "auto" | "direct" (the GPU reads the lists and writes the forces in
    place in host memory; a GPU with pageable host memory access, e.g. on Grace) | "staged"
    (pinned copies)."""

    def __init__(self, model: DP, pair_coeff: Sequence[int], eatom_grouped: bool = True,
                 host_access: str = "auto"):
        at = list(model.cfg.atom_type)
        for z in pair_coeff:
            if z not in at:   # pair_matpl.cpp:296-299
                raise _lib.MatplError("This element is not included in the machine learning "
                                      f"force field: {z}")
        self.model = model
        self.type_to_model = [at.index(int(z)) for z in pair_coeff]
        self.ntypes_lmp = len(self.type_to_model)
        t2m = (ctypes.c_int * self.ntypes_lmp)(*self.type_to_model)
        present = list(range(model.cfg.ntypes))
        self._mstruct = model._model_struct(present)
        modes = {"auto": _lib.LMP_AUTO, "staged": _lib.LMP_STAGED, "direct": _lib.LMP_DIRECT}
        if host_access not in modes:
            raise _lib.MatplError(f"host_access is one of {list(modes)}")
        h = ctypes.c_void_p()
        lib = _lib.load()
        check(lib.matpl_lammps_dp_create(model.code, ctypes.byref(self._mstruct), self.ntypes_lmp,
                                         ctypes.cast(t2m, ctypes.c_void_p), int(eatom_grouped),
                                         modes[host_access], ctypes.byref(h)),
              "matpl_lammps_dp_create")
        self._h = h
        self.host_access = {_lib.LMP_STAGED: "staged", _lib.LMP_DIRECT: "direct"}[
            lib.matpl_lammps_dp_host_access(h)]
        self.models = [model]
        self._structs = [self._mstruct]

    def add_model(self, model: DP):
        """Another model for the deviation (``pair_style matpl m1.pt m2.pt ...``): same type
        count, maxNeighborNum and Rmax as the first, any weights and precision form that
        matches the first's dtype."""
        if model.code != self.models[0].code:
            raise _lib.MatplError("all models of one pair style use the same precision form")
        st = model._model_struct(list(range(model.cfg.ntypes)))
        check(_lib.load().matpl_lammps_dp_add_model(self._h, ctypes.byref(st)),
              "matpl_lammps_dp_add_model")
        self.models.append(model)
        self._structs.append(st)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().matpl_lammps_dp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def compute(self, x: np.ndarray, type_: np.ndarray, nlocal: int, nghost: int,
                ilist: np.ndarray, numneigh: np.ndarray, firstneigh: np.ndarray,
                eflag_atom: bool = False, f_out: Optional[np.ndarray] = None) -> Dict:
        """x [nall, 3] f64 (atom->x), type_ [nall] int32 1-based, ilist [inum] int32,
        numneigh [nlocal] int32, firstneigh [nlocal] uint64 host addresses of each atom's
        int32 list (LAMMPS' int**).  Returns dict(f [nall, 3], eng, virial [6], eatom, min_rsq);
        raises like the reference when two atoms are closer than sqrt(0.61)."""
        nall = nlocal + nghost
        x = _np(x, np.float64).reshape(nall, 3)
        type_ = _np(type_, np.int32)
        ilist = _np(ilist, np.int32)
        numneigh = _np(numneigh, np.int32)
        firstneigh = _np(firstneigh, np.uint64)
        f = f_out if f_out is not None else np.zeros((nall, 3), dtype=np.float64)
        eng = ctypes.c_double(0.0)
        vir = np.zeros(6, dtype=np.float64)
        eatom = np.zeros(len(ilist), dtype=np.float64) if eflag_atom else None
        mn = ctypes.c_double(0.0)
        c = ctypes.c_void_p
        check(_lib.load().matpl_lammps_dp_compute(
            self._h, int(nlocal), int(nghost), len(ilist), ilist.ctypes.data_as(c),
            numneigh.ctypes.data_as(c), firstneigh.ctypes.data_as(c), x.ctypes.data_as(c),
            type_.ctypes.data_as(c), f.ctypes.data_as(c), ctypes.cast(ctypes.byref(eng), c),
            vir.ctypes.data_as(c), eatom.ctypes.data_as(c) if eatom is not None else None,
            ctypes.cast(ctypes.byref(mn), c)), "matpl_lammps_dp_compute")
        if len(ilist) and mn.value < MIN_RSQ:
            raise _lib.MatplError(f"there are two atoms too close, min_dR_all = {mn.value}")
        return {"f": f, "eng": eng.value, "virial": vir, "eatom": eatom, "min_rsq": mn.value}


@_lib.on_device
def _compute_models(pair: PairMATPL, nmodels, x, type_, nlocal, nghost, ilist, numneigh,
                    firstneigh, eflag_atom):
    nall = nlocal + nghost
    x = _np(x, np.float64).reshape(nall, 3)
    type_ = _np(type_, np.int32)
    ilist = _np(ilist, np.int32)
    numneigh = _np(numneigh, np.int32)
    firstneigh = _np(firstneigh, np.uint64)
    f = np.zeros((nmodels, nall, 3), dtype=np.float64)
    eng = np.zeros(nmodels, dtype=np.float64)
    vir = np.zeros((nmodels, 6), dtype=np.float64)
    eatom = np.zeros((nmodels, len(ilist)), dtype=np.float64) if eflag_atom else None
    mn = ctypes.c_double(0.0)
    c = ctypes.c_void_p
    check(_lib.load().matpl_lammps_dp_compute_models(
        pair._h, nmodels, int(nlocal), int(nghost), len(ilist), ilist.ctypes.data_as(c),
        numneigh.ctypes.data_as(c), firstneigh.ctypes.data_as(c), x.ctypes.data_as(c),
        type_.ctypes.data_as(c), f.ctypes.data_as(c), eng.ctypes.data_as(c),
        vir.ctypes.data_as(c), eatom.ctypes.data_as(c) if eatom is not None else None,
        ctypes.cast(ctypes.byref(mn), c)), "matpl_lammps_dp_compute_models")
    if len(ilist) and mn.value < MIN_RSQ:
        raise _lib.MatplError(f"there are two atoms too close, min_dR_all = {mn.value}")
    return {"f": f, "eng": eng, "virial": vir, "eatom": eatom, "min_rsq": mn.value}


def compute_models(pair: PairMATPL, x, type_, nlocal, nghost, ilist, numneigh, firstneigh,
                   eflag_atom: bool = True) -> Dict:
    """Every model of the pair style on one slot conversion: f [K, nall, 3], eng [K],
    virial [K, 6], eatom [K, inum] (the f_n / e_atom_n of pair_matpl.cpp:951-963)."""
    return _compute_models(pair, len(pair.models), x, type_, nlocal, nghost, ilist, numneigh,
                           firstneigh, eflag_atom)


def model_deviation(f_n: np.ndarray, e_n: np.ndarray) -> Tuple[float, ...]:
    """PairMATPL::calc_max_error (pair_matpl.cpp:385-483) after the ghost rows are folded:
    f_n [K, nlocal, 3], e_n [K, nlocal] -> (max over atoms of the RMS force deviation, max and
    min per-model force deviation, the same three for Ei), the model_devi.out columns."""
    f_n = np.asarray(f_n, dtype=np.float64)
    e_n = np.asarray(e_n, dtype=np.float64)
    K = f_n.shape[0]
    ferr = f_n - f_n.mean(0)
    fe = np.sqrt((ferr * ferr).sum(-1))                 # [K, nlocal]
    eerr = np.abs(e_n - e_n.mean(0))
    max_mean_f = float(np.sqrt((fe * fe).sum(0) / K).max())
    max_mean_e = float(np.sqrt((eerr * eerr).sum(0) / K).max())
    return (max_mean_f, float(fe.max()), float(fe.min()), max_mean_e, float(eerr.max()),
            float(eerr.min()))


@_lib.on_device
def lammps_dp_neighbors(ilist: torch.Tensor, jstart: torch.Tensor, jflat: torch.Tensor,
                        x: torch.Tensor, type_: torch.Tensor, type_to_model: torch.Tensor,
                        ntypes: int, m: int, rcut: float, dtype=torch.float64,
                        err: Optional[torch.Tensor] = None) -> Dict[str, torch.Tensor]:
    """``matpl_lammps_dp_neighbors`` on device tensors (the slot conversion alone):
    list_neigh [1, inum, S] int32, ImageDR [1, inum, S, 4], Imagetype_map [inum] int32,
    min_rsq [1] f64, err [1] int32."""
    dev = x.device
    inum = ilist.numel()
    nall = x.shape[0]
    S = ntypes * m
    out = {"list_neigh": torch.empty(1, inum, S, dtype=torch.int32, device=dev),
           "ImageDR": torch.empty(1, inum, S, 4, dtype=dtype, device=dev),
           "Imagetype_map": torch.empty(inum, dtype=torch.int32, device=dev),
           "min_rsq": torch.empty(1, dtype=torch.float64, device=dev),
           "err": err if err is not None else torch.zeros(1, dtype=torch.int32, device=dev)}
    code = _lib.MATPL_F64 if dtype == torch.float64 else _lib.MATPL_F32
    jf = jflat if jflat.numel() else torch.zeros(1, dtype=torch.int32, device=dev)
    check(_lib.load().matpl_lammps_dp_neighbors(
        inum, nall, ptr(ilist), ptr(jstart), ptr(jf), ptr(x), ptr(type_), ptr(type_to_model),
        type_to_model.numel(), ntypes, m, float(rcut), code, ptr(out["list_neigh"]),
        ptr(out["ImageDR"]), ptr(out["Imagetype_map"]), ptr(out["min_rsq"]), ptr(out["err"]),
        torch.cuda.current_stream(dev).cuda_stream), "matpl_lammps_dp_neighbors")
    return out


def lammps_system(lattice: np.ndarray, cart: np.ndarray, ltype: np.ndarray, cutneigh: float,
                  seed: int = 0, shuffle: bool = True) -> Dict[str, np.ndarray]:
    """Local atoms (wrapped into the cell), ghost atoms = periodic images whose fractional
    coordinates lie within cutneigh / (cell width) of the cell (the triclinic ghost rule of
    LAMMPS), and a full neighbor list (every j != i within cutneigh) per local atom in random
    order.  lattice rows are the cell vectors; ltype 1-based LAMMPS types.  Returns x [nall, 3],
    type [nall], nlocal, nghost, owner [nall] (local atom each row images), ilist, numneigh,
    jstart [nlocal+1], jflat (CSR, row ii = atom ii)."""
    from scipy.spatial import cKDTree
    lat = np.asarray(lattice, dtype=np.float64)
    frac = np.mod(np.asarray(cart, dtype=np.float64) @ np.linalg.inv(lat), 1.0)
    frac[frac >= 1.0] = 0.0
    n = frac.shape[0]
    vol = abs(np.linalg.det(lat))
    width = np.array([vol / np.linalg.norm(np.cross(lat[(d + 1) % 3], lat[(d + 2) % 3]))
                      for d in range(3)])
    cg = cutneigh / width
    K = np.ceil(cg).astype(int)
    xs, owners = [frac @ lat], [np.arange(n)]
    for a in range(-K[0], K[0] + 1):
        for b in range(-K[1], K[1] + 1):
            for c in range(-K[2], K[2] + 1):
                if a == 0 and b == 0 and c == 0:
                    continue
                fs = frac + np.array([a, b, c], dtype=np.float64)
                keep = np.all((fs >= -cg) & (fs < 1.0 + cg), axis=1)
                if keep.any():
                    xs.append(fs[keep] @ lat)
                    owners.append(np.nonzero(keep)[0])
    x = np.concatenate(xs)
    owner = np.concatenate(owners)
    types = np.asarray(ltype, dtype=np.int32)[owner]
    tree = cKDTree(x)
    lists = tree.query_ball_point(x[:n], r=cutneigh, return_sorted=False)
    cnt = np.array([len(l) - 1 for l in lists], dtype=np.int32)
    rows = np.repeat(np.arange(n), cnt + 1)
    flat = np.concatenate([np.asarray(l, dtype=np.int64) for l in lists])
    keep = flat != rows
    rows, flat = rows[keep], flat[keep]
    rng = np.random.default_rng(seed)
    key = rng.random(flat.size) if shuffle else flat.astype(np.float64)
    order = np.lexsort((key, rows))
    jflat = flat[order].astype(np.int32)
    jstart = np.zeros(n + 1, dtype=np.int64)
    jstart[1:] = np.cumsum(cnt)
    return {"x": np.ascontiguousarray(x), "type": types, "nlocal": n,
            "nghost": int(x.shape[0] - n), "owner": owner, "ilist": np.arange(n, dtype=np.int32),
            "numneigh": cnt, "jstart": jstart, "jflat": jflat}


def firstneigh_of(system: Dict[str, np.ndarray]) -> np.ndarray:
    """LAMMPS-style per-atom list addresses (int**) into the system's jflat array."""
    jf = system["jflat"]
    return (np.uint64(jf.ctypes.data) + 4 * system["jstart"][:-1].astype(np.uint64)).astype(
        np.uint64)


def fold_ghosts(f: np.ndarray, owner: np.ndarray, nlocal: int) -> np.ndarray:
    """What LAMMPS' reverse communication does with ghost forces: add each ghost row to the
    local atom it images."""
    out = f[:nlocal].copy()
    np.add.at(out, owner[nlocal:], f[nlocal:])
    return out
