"""ORACLE — test infrastructure only (see ``oracle/__init__.py``).

numpy glue around ``lammps_neigh.c``, the restatement of ``PairMATPL::generate_neighdata``
(``src/lmps/lammps-libtorch/MATPL/pair_matpl.cpp:522-616``), and the rest of the reference's
DP pair step (``pair_matpl.cpp:893-996``) on top of the DP oracle: the TorchScript model's
forward with ghost rows (``src/model/dp_dp_script.py:137-185, 387-428``), the forces of local
and ghost atoms, the Voigt virial ``[0, 4, 8, 1, 2, 5]`` and Ei in the model's type-grouped
order.
"""
import ctypes

import numpy as np
import torch

from . import build as _build

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
        f = _lib.oracle_lammps_dp_neighdata
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 6 + [ctypes.c_int, ctypes.c_int,
                                                              ctypes.c_double] + [ctypes.c_void_p] * 4
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def neighdata(ilist, jstart, jflat, x, type_, type_to_model, nt, m, cutoff):
    """Returns (list_neigh [1, inum, nt*m] int32, ImageDR [1, inum, nt*m, 4] f64,
    type_map [inum] int32, min_rsq, overflow)."""
    ilist = np.ascontiguousarray(ilist, dtype=np.int32)
    jstart = np.ascontiguousarray(jstart, dtype=np.int64)
    jflat = np.ascontiguousarray(jflat, dtype=np.int32)
    x = np.ascontiguousarray(x, dtype=np.float64)
    type_ = np.ascontiguousarray(type_, dtype=np.int32)
    t2m = np.ascontiguousarray(type_to_model, dtype=np.int32)
    inum = ilist.shape[0]
    S = nt * m
    ln = np.zeros((1, inum, S), dtype=np.int32)
    dr = np.zeros((1, inum, S, 4), dtype=np.float64)
    tm = np.zeros(inum, dtype=np.int32)
    mn = np.zeros(1, dtype=np.float64)
    jf = jflat if jflat.size else np.zeros(1, dtype=np.int32)
    ov = _load().oracle_lammps_dp_neighdata(inum, _p(ilist), _p(jstart), _p(jf), _p(x), _p(type_),
                                            _p(t2m), nt, m, float(cutoff), _p(ln), _p(dr), _p(tm),
                                            _p(mn))
    return ln, dr, tm, float(mn[0]), bool(ov)


def pair_compute(cfg, params, davg, dstd, type_to_model, nlocal, nghost, ilist, jstart, jflat, x,
                 type_):
    """The reference's DP pair step on the CPU: generate_neighdata, then the DP forward with
    nghost (the TorchScript model's arithmetic, ``dp_oracle.dp_eval`` with the CPU virial),
    then what ``compute`` keeps.  Returns dict(f [nall, 3], eng, virial [6], eatom [inum]
    (type-grouped, as pair_matpl.cpp:1000 stores it), eatom_atom [inum], min_rsq)."""
    from . import dp_oracle
    ln, dr, tm, mn, ov = neighdata(ilist, jstart, jflat, x, type_, type_to_model, cfg.ntypes,
                                   cfg.maxNeighborNum, cfg.Rmax)
    if ov:
        raise RuntimeError("a type block holds more than maxNeighborNum neighbors")
    atom_type = torch.tensor([cfg.atom_type[t] for t in type_to_model])
    out = dp_oracle.dp_eval(cfg, params, davg, dstd, torch.tensor(ln), torch.tensor(tm),
                            atom_type, torch.tensor(dr), nghost, virial_convention="cpu")
    V = out["Virial"][0].detach().numpy()
    return {"f": out["Force"][0].detach().numpy(), "eng": float(out["Etot"].detach().sum()),
            "virial": V[[0, 4, 8, 1, 2, 5]], "eatom": out["Ei"][0].detach().numpy(),
            "eatom_atom": out["Ei_atom"][0].detach().numpy(), "min_rsq": mn,
            "list_neigh": ln, "image_dr": dr, "type_map": tm}
