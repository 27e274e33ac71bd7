"""ORACLE — test infrastructure only (see ``oracle/__init__.py``).

numpy glue around ``neighconst.c`` that reproduces what MatPL's loader hands the model:
``src/pre_data/dpuni_data_loader.py:595-650`` (``find_neighbore``) and ``:652-716``
(``compute_Ri``'s ``Rij`` column), i.e. ``list_neigh`` [images, natoms, ntypes*m] int32
(1-based, 0 = empty) and ``ImageDR`` [images, natoms, ntypes*m, 4] = (r, dx, dy, dz).
"""
import ctypes

import numpy as np

from . import build as _build

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
        f = _lib.matpl_oracle_find_neighbore
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                      ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_void_p]
        g = _lib.matpl_oracle_image_dr
        g.restype = None
        g.argtypes = [ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return _lib


class NeighborOverflow(RuntimeError):
    """Raised where NeighConst.f90:75-78 prints "maxNeighborNum too small" and stops."""


def find_neighbore(type_maps, frac_position, lattice, ntypes, m_neigh, Rc_M, Rc_type):
    """Oracle neighbor search for one or more images.

    type_maps: [natoms] 0-based type index of each atom (the loader adds 1 before Fortran).
    frac_position: [images, natoms, 3] or [natoms, 3] fractional coordinates.
    lattice: [images, 3, 3] or [3, 3], rows are lattice vectors.
    Returns (list_neigh int32 [images, natoms, ntypes*m], ImageDR f64 [images, natoms, ntypes*m, 4]).
    """
    lib = _load()
    pos = np.ascontiguousarray(np.array(frac_position, dtype=np.float64).reshape(-1, len(type_maps), 3))
    images, natoms = pos.shape[0], pos.shape[1]
    lat = np.ascontiguousarray(np.array(lattice, dtype=np.float64).reshape(images, 3, 3))
    tmap = np.ascontiguousarray(np.asarray(type_maps, dtype=np.int32) + 1)
    rct = np.ascontiguousarray(np.broadcast_to(np.asarray(Rc_type, dtype=np.float64), (ntypes,)).copy())
    S = ntypes * m_neigh
    ln = np.zeros((images, natoms, S), dtype=np.int32)
    dr = np.zeros((images, natoms, S, 3), dtype=np.float64)
    rc = lib.matpl_oracle_find_neighbore(images, lat.ctypes.data, pos.ctypes.data, ntypes, natoms,
                                         m_neigh, float(Rc_M), rct.ctypes.data, tmap.ctypes.data,
                                         ln.ctypes.data, dr.ctypes.data)
    if rc == 1:
        raise NeighborOverflow(f"maxNeighborNum too small {m_neigh}")
    if rc != 0:
        raise RuntimeError(f"oracle neighbor search failed ({rc})")
    idr = np.zeros((images, natoms, S, 4), dtype=np.float64)
    lib.matpl_oracle_image_dr(images * natoms * S, ln.ctypes.data, dr.ctypes.data, idr.ctypes.data)
    return ln, idr


def env_sums(cfg, list_neigh, image_dr, type_map):
    """ORACLE of matpl_env_stats: [B, ntypes, 8] sums of Ri_c and Ri_c^2 (c = 0..3) over the
    slots of each centre type, Ri = vv(r) (1/r, x/r^2, y/r^2, z/r^2) with r, r^2 formed from the
    pair vector like calc_stat + smooth (src/pre_data/dpuni_data_loader.py:436-534)."""
    ln = np.asarray(list_neigh)
    dr = np.asarray(image_dr, dtype=np.float64)
    B, N, S = ln.shape
    tm = np.asarray(type_map)
    out = np.zeros((B, cfg.ntypes, 8))
    mask = ln > 0
    xyz = dr[..., 1:]
    r2 = (xyz * xyz).sum(-1)
    r2s = np.where(mask, r2, 1.0)
    r = r2s / np.sqrt(r2s)
    u = (r - cfg.Rmin) / (cfg.Rmax - cfg.Rmin)
    vv = np.where(r < cfg.Rmin, 1.0, np.where(r < cfg.Rmax, u ** 3 * (-6 * u * u + 15 * u - 10) + 1,
                                              0.0))
    Ri = np.stack([vv / r, vv * xyz[..., 0] / r2s, vv * xyz[..., 1] / r2s, vv * xyz[..., 2] / r2s],
                  -1)
    Ri = np.where(mask[..., None], Ri, 0.0)
    for b in range(B):
        for t in range(cfg.ntypes):
            sel = Ri[b][tm == t].reshape(-1, 4)
            out[b, t, 0::2] = sel.sum(0)
            out[b, t, 1::2] = (sel * sel).sum(0)
    return out

