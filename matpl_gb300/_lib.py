"""ctypes binding of ``libmatpl_gb300.so`` (the C ABI declared in ``include/matpl_gb300.h``).

The library is built in-tree by ``matpl_gb300.build``.  There is no fallback: when the library
is missing or a call fails, a ``MatplError`` is raised.
"""
import ctypes
import functools
import os

import torch

from . import build as _build

MATPL_F32, MATPL_F64, MATPL_MIXED, MATPL_MIXED_FAST, MATPL_MIXED_TANHF = 0, 1, 2, 3, 4
KERR_NEIGHBOR_OVERFLOW = 1
KERR_BAD_TYPE = 2
KERR_TIMEOUT = 3
KERR_BAD_BOX = 4
KERR_BAD_COUNT = 5
KERR_TABLE_RANGE = 6
LMP_AUTO, LMP_STAGED, LMP_DIRECT = 0, 1, 2

_c = ctypes
_vp, _i, _d, _sz = _c.c_void_p, _c.c_int, _c.c_double, _c.c_size_t


class MatplDpModel(ctypes.Structure):
    """Mirror of ``matpl_dp_model``."""
    _fields_ = [("ntypes", _i), ("m", _i), ("npresent", _i), ("present", _i * 8),
                ("rmin", _d), ("rmax", _d), ("params", _vp), ("davg", _vp), ("dstd", _vp),
                ("err_dev", _vp), ("ctable", _vp), ("ctab_rows", _i), ("ctab_order", _i),
                ("ctab_dx", _d), ("ctab_smin", _d), ("ctab_smax", _d)]


class MatplNepModel(ctypes.Structure):
    """Mirror of ``matpl_nep_model``."""
    _fields_ = [("ntypes", _i), ("n_max_radial", _i), ("basis_radial", _i),
                ("n_max_angular", _i), ("basis_angular", _i), ("l_max_3b", _i), ("l_max_4b", _i),
                ("l_max_5b", _i), ("neuron", _i), ("train_2b", _i), ("cutoff_radial", _d),
                ("cutoff_angular", _d), ("params", _vp), ("err_dev", _vp)]


_ll = _c.c_longlong

# name -> (restype, argtypes)
SIGNATURES = {
    "matpl_last_error": (_c.c_char_p, []),
    "matpl_version": (_i, []),
    "matpl_profile_begin": (_i, [_i]),
    "matpl_profile_collect": (_i, [_i, _c.c_char_p, _i, _c.POINTER(_d), _c.POINTER(_i),
                                   _c.POINTER(_i)]),
    "matpl_calc_force": (_i, [_i, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp, _vp]),
    "matpl_calc_virial": (_i, [_i, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp, _vp, _vp]),
    "matpl_calc_force_grad": (_i, [_i, _vp, _vp, _vp, _i, _i, _i, _i, _vp, _vp]),
    "matpl_calc_virial_grad": (_i, [_i, _vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp]),
    "matpl_calc_compress": (_i, [_i, _vp, _vp, _c.c_longlong, _i, _i, _vp, _vp]),
    "matpl_calc_compress_grad": (_i, [_i, _vp, _vp, _vp, _c.c_longlong, _i, _i, _vp, _vp]),
    "matpl_neighbor_workspace_bytes": (_sz, [_i, _i]),
    "matpl_neighbor_build": (_i, [_i, _i, _i, _i, _d, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp,
                                  _vp, _vp, _sz, _vp]),
    "matpl_neighbor_build_noalloc": (_i, [_i, _i, _i, _i, _d, _vp, _vp, _vp, _vp, _i, _vp, _vp,
                                          _vp, _vp, _vp]),
    "matpl_neighbor_build_occupied": (_i, [_i, _i, _i, _i, _d, _vp, _vp, _vp, _vp, _i, _vp, _vp,
                                           _vp, _vp, _vp, _sz, _vp]),
    "matpl_env_mat": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _d, _d, _vp, _vp, _vp]),
    "matpl_dp_param_count": (_sz, [_i]),
    "matpl_dp_workspace_bytes": (_sz, [_i, _i, _i]),
    "matpl_dp_eval": (_i, [_i, _c.POINTER(MatplDpModel), _i, _i, _i, _i, _vp, _vp, _vp, _vp,
                           _vp, _vp, _vp, _vp, _sz, _vp]),
    "matpl_dp_eval_occupied": (_i, [_i, _c.POINTER(MatplDpModel), _i, _i, _i, _i, _vp, _vp,
                                    _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "matpl_dp_set_wait_limit": (_i, [_i]),
    "matpl_dp_set_tuning": (_i, [_i, _i]),
    "matpl_dp_get_tuning": (_i, [_c.POINTER(_i), _c.POINTER(_i)]),
    "matpl_dp_dual_forward": (_i, [_i, _c.POINTER(MatplDpModel), _i, _i, _i, _vp, _vp, _vp,
                                   _vp, _vp, _vp, _vp, _vp]),
    "matpl_dp_dual_backward": (_i, [_i, _c.POINTER(MatplDpModel), _i, _i, _i, _vp, _vp, _vp,
                                    _vp, _vp, _vp, _vp, _vp, _vp]),
    "matpl_nep_neighbor_workspace_bytes": (_sz, [_i, _ll]),
    "matpl_nep_neighbor": (_i, [_i, _ll, _vp, _vp, _vp, _vp, _vp, _d, _d, _i, _i, _i, _vp, _vp,
                                _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "matpl_nep_maxneigh": (_i, [_i, _ll, _vp, _vp, _vp, _vp, _vp, _d, _d, _i, _vp, _i, _vp, _vp,
                                _vp, _vp, _sz, _vp]),
    "matpl_dp_pad_workspace_bytes": (_sz, [_i]),
    "matpl_dp_pad_forward": (_i, [_i, _c.POINTER(MatplDpModel), _i, _i, _i] + [_vp] * 6 +
                             [_sz, _vp]),
    "matpl_dp_pad_backward": (_i, [_i, _c.POINTER(MatplDpModel), _i, _i, _i] + [_vp] * 5 +
                              [_sz, _vp]),
    "matpl_dp_fit_dual_workspace_bytes": (_sz, [_i, _ll]),
    "matpl_dp_fit_dual": (_i, [_i, _ll] + [_vp] * 8 + [_vp, _sz, _vp]),
    "matpl_nep_skin_update": (_i, [_i, _ll, _vp, _vp, _vp, _vp, _vp, _d, _d, _i] + [_vp] * 9 +
                              [_sz, _vp]),
    "matpl_nep_skin_filter_compact": (_i, [_ll, _d, _d, _i, _i, _i] + [_vp] * 12),
    "matpl_nep_skin_filter": (_i, [_i, _ll, _vp, _d, _d, _i, _i, _i, _i] + [_vp] * 10 +
                              [_sz, _vp]),
    "matpl_nep_param_count": (_sz, [_c.POINTER(MatplNepModel)]),
    "matpl_nep_workspace_bytes": (_sz, [_i, _i, _ll]),
    "matpl_nep_eval": (_i, [_i, _c.POINTER(MatplNepModel), _i, _ll, _vp, _vp, _i, _vp, _vp, _vp,
                            _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "matpl_nep_eval_compact": (_i, [_i, _c.POINTER(MatplNepModel), _i, _ll, _vp, _vp, _i, _vp,
                                    _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz,
                                    _vp]),
    "matpl_nep_descriptor": (_i, [_i, _c.POINTER(MatplNepModel), _i, _ll, _vp, _vp, _i, _vp, _vp,
                                  _vp, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "matpl_env_stats": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _d, _d, _vp, _vp, _vp]),
    "matpl_nep_feat_op": (_i, [_i] * 11 + [_d] + [_vp] * 5 + [_ll, _vp, _vp, _ll] + [_vp] * 4),
    "matpl_nep_cgrad": (_i, [_i] * 6 + [_vp, _vp, _ll, _vp, _vp, _vp, _vp]),
    "matpl_dp_desc_dual": (_i, [_i, _ll, _i] + [_vp] * 6),
    "matpl_dp_desc_dual_grad": (_i, [_i, _ll, _i] + [_vp] * 8),
    "matpl_nep_force_virial": (_i, [_i] * 4 + [_vp] * 8),
    "matpl_nep_zbl": (_i, [_i, _i, _ll, _i, _i] + [_vp] * 4 + [_i, _vp, _vp, _d] + [_vp] * 6),
    "matpl_nep_force_virial_grad": (_i, [_i] * 4 + [_vp] * 8),
    "matpl_lammps_dp_neighbors": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _i,
                                       _vp, _vp, _vp, _vp, _vp, _vp]),
    "matpl_lammps_dp_create": (_i, [_i, _c.POINTER(MatplDpModel), _i, _vp, _i, _i,
                                    _c.POINTER(_vp)]),
    "matpl_lammps_dp_host_access": (_i, [_vp]),
    "matpl_lammps_dp_compute": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                     _vp, _vp]),
    "matpl_lammps_dp_destroy": (None, [_vp]),
    "matpl_lammps_dp_add_model": (_i, [_vp, _c.POINTER(MatplDpModel)]),
    "matpl_lammps_dp_num_models": (_i, [_vp]),
    "matpl_lammps_dp_compute_models": (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp,
                                            _vp, _vp, _vp, _vp]),
    "matpl_md_drift": (_i, [_i, _d, _d, _vp, _vp, _vp, _vp, _vp, _vp]),
    "matpl_md_skin_build": (_i, [_i, _i, _i, _i, _d, _vp, _vp, _i] + [_vp] * 12),
    "matpl_md_skin_filter": (_i, [_i, _i, _i, _i, _i, _d] + [_vp] * 11),
    "matpl_md_kick": (_i, [_i, _i, _i, _d, _d] + [_vp] * 10),
}


class MatplError(RuntimeError):
    pass


_LIB = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the native library and bind every entry point."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise MatplError(f"native library not built: {path} (run matpl_gb300.build.build())")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def check(status: int, what: str):
    if status != 0:
        msg = load().matpl_last_error().decode(errors="replace")
        raise MatplError(f"{what} failed (status {status}): {msg}")


def profile_begin(max_launches: int = 65536):
    check(load().matpl_profile_begin(max_launches), "matpl_profile_begin")


def profile_collect():
    """{kernel: (total_ms, launches)} for launches since profile_begin()."""
    n = 64
    names = ctypes.create_string_buffer(n * 64)
    ms = (ctypes.c_double * n)()
    cnt = (ctypes.c_int * n)()
    nout = ctypes.c_int()
    check(load().matpl_profile_collect(n, names, 64, ms, cnt, ctypes.byref(nout)),
          "matpl_profile_collect")
    out = {}
    for k in range(nout.value):
        nm = names.raw[k * 64:(k + 1) * 64].split(b"\0", 1)[0].decode()
        out[nm] = (ms[k], cnt[k])
    return out


def ptr(t) -> int:
    """Device pointer of a torch tensor (None -> NULL)."""
    return 0 if t is None else t.data_ptr()


def _cuda_devices(objs, found):
    for o in objs:
        if isinstance(o, torch.Tensor):
            if o.is_cuda:
                found.add(o.device.index)
        elif isinstance(o, (list, tuple)):
            _cuda_devices(o, found)


def on_device(fn):
    """Run ``fn`` with the device of its CUDA tensor arguments current.

    The C library launches on the current device (and torch's current stream of the tensors'
    device is passed to it), so every wrapper that calls into it goes through this: tensors
    spread over several GPUs are refused, and the GPU that holds them is made current for the
    duration of the call (a no-op when it already is)."""
    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        found = set()
        _cuda_devices(args, found)
        _cuda_devices(kwargs.values(), found)
        if not found:
            return fn(*args, **kwargs)
        if len(found) > 1:
            raise MatplError(f"{fn.__qualname__}: CUDA tensors on several devices "
                             f"{sorted(found)}; put every argument on one GPU")
        with torch.cuda.device(found.pop()):
            return fn(*args, **kwargs)
    return wrapper
