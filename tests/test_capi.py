"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and exports every
function that include/matpl_gb300.h declares; host-side argument checks; the ctypes mirrors
agree with the header's struct layouts and codes; host-side packing logic."""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest
import torch

from matpl_gb300 import _lib, dp, params as P

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(REPO, "include", "matpl_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(matpl_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = header_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), f"{n} declared in the header but not exported"
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_version_and_error_string():
    lib = _lib.load()
    assert lib.matpl_version() >= 1
    assert isinstance(lib.matpl_last_error(), bytes)


def test_host_side_validation_needs_no_gpu():
    """Argument errors are caught on the host before any CUDA call."""
    lib = _lib.load()
    st = lib.matpl_calc_force(7, None, None, None, None, 1, 1, 1, 0, None, None)
    assert st == 2  # MATPL_ERR_DTYPE
    assert b"f32" in lib.matpl_last_error()
    st = lib.matpl_neighbor_build(1, 4, 1, 10, 6.0, (ctypes.c_double * 1)(6.0), None, None, None,
                                  0, None, None, None, None, None, 0, None)
    assert st in (1, 3)  # missing err_dev / workspace
    m = _lib.MatplDpModel()
    m.ntypes, m.m, m.npresent = 1, 100, 0
    st = lib.matpl_dp_eval(1, ctypes.byref(m), 1, 1, 100, 0, None, None, None, None, None, None,
                           None, None, 0, None)
    assert st == 1


def test_training_and_nep_entry_points_validate_on_the_host():
    """The training / NEP entry points refuse bad dtypes and sizes before any CUDA call."""
    lib = _lib.load()
    err = ctypes.c_int(0)
    st = lib.matpl_nep_zbl(9, 1, 10, 4, 1, None, None, None, None, 2, None, None, 2.0, None, None,
                           None, None, ctypes.byref(err), None)
    assert st == 2 and b"dtype" in lib.matpl_last_error()
    st = lib.matpl_nep_zbl(0, 1, 10, 4, 1, None, None, None, None, 2, None, None, -1.0, None,
                           None, None, None, ctypes.byref(err), None)
    assert st == 1
    st = lib.matpl_dp_desc_dual(0, 10, 0, None, None, None, None, None, None)
    assert st == 1 and b"m2" in lib.matpl_last_error()
    st = lib.matpl_dp_desc_dual_grad(1, 10, 26, None, None, None, None, None, None, None, None)
    assert st == 1
    st = lib.matpl_nep_cgrad(0, 2, 10, 2, 4, 8, None, None, 4, None, None, ctypes.byref(err), None)
    assert st == 1 and b"part" in lib.matpl_last_error()
    st = lib.matpl_nep_force_virial(0, 10, 4, 0, None, None, None, None, None, None,
                                    ctypes.byref(err), None)
    assert st == 1
    m = _lib.MatplDpModel()
    m.ntypes, m.m, m.npresent, m.present[0] = 1, 100, 1, 0
    m.ctable, m.ctab_order, m.ctab_rows, m.ctab_dx = 1, 4, 10, 0.01      # order must be 3 or 5
    ws = ctypes.create_string_buffer(1 << 20)
    st = lib.matpl_dp_eval(1, ctypes.byref(m), 1, 1, 100, 0, None, None, None, None, None, None,
                           None, ws, len(ws), None)
    assert st == 1 and b"compressed" in lib.matpl_last_error()


def test_empty_sizes_and_null_pointers_are_handled_on_the_host():
    """Empty inputs return MATPL_OK before any CUDA call; a NULL pointer that the sizes would
    make a kernel read or write is refused (MATPL_ERR_INVALID) instead of reaching the GPU."""
    lib = _lib.load()
    err = ctypes.c_int(0)
    OK, INVALID = 0, 1
    assert lib.matpl_calc_force(0, None, None, None, None, 2, 0, 5, 0, None, None) == OK
    assert lib.matpl_calc_force(0, None, None, None, None, 1, 3, 5, 0, None, None) == INVALID
    assert b"null" in lib.matpl_last_error()
    assert lib.matpl_calc_virial(1, None, None, None, None, 0, 3, 5, 0, None, None, None) == OK
    assert lib.matpl_calc_virial(1, None, None, None, None, 1, 3, 5, 0, None, None,
                                 None) == INVALID
    assert lib.matpl_calc_force_grad(0, None, None, None, 1, 0, 5, 0, None, None) == OK
    assert lib.matpl_calc_force_grad(0, None, None, None, 1, 3, 5, 0, None, None) == INVALID
    assert lib.matpl_calc_virial_grad(0, None, None, None, None, 1, 3, 0, None, None) == OK
    assert lib.matpl_calc_virial_grad(0, None, None, None, None, 1, 3, 5, None, None) == INVALID
    assert lib.matpl_env_mat(1, 1, 0, 200, None, None, None, None, 0.5, 6.0, None, None,
                             None) == OK
    assert lib.matpl_env_mat(1, 1, 4, 200, None, None, None, None, 0.5, 6.0, None, None,
                             None) == INVALID
    assert lib.matpl_calc_compress(1, None, None, 0, 25, 6, None, None) == OK
    assert lib.matpl_calc_compress(1, None, None, 10, 25, 6, None, None) == INVALID
    assert lib.matpl_calc_compress_grad(1, None, None, None, 0, 25, 4, None, None) == OK
    assert lib.matpl_calc_compress_grad(1, None, None, None, 10, 25, 4, None, None) == INVALID
    assert lib.matpl_dp_desc_dual(0, 0, 16, None, None, None, None, None, None) == OK
    assert lib.matpl_dp_desc_dual_grad(1, 0, 16, None, None, None, None, None, None, None,
                                       None) == OK
    assert lib.matpl_nep_zbl(1, 1, 0, 4, 1, None, None, None, None, 2, None, None, 2.0, None, None,
                             None, None, ctypes.byref(err), None) == OK
    assert lib.matpl_nep_zbl(1, 1, 5, 4, 1, None, None, None, None, 2, None, None, 2.0, None, None,
                             None, None, ctypes.byref(err), None) == INVALID
    assert lib.matpl_nep_force_virial_grad(0, 0, 4, 1, None, None, None, None, None, None,
                                           ctypes.byref(err), None) == OK
    assert err.value == 0
    m = _lib.MatplDpModel()
    m.ntypes, m.m, m.npresent, m.present[0] = 1, 100, 1, 0
    ws = ctypes.create_string_buffer(1 << 20)
    assert lib.matpl_dp_eval(1, ctypes.byref(m), 0, 4, 100, 0, None, None, None, None, None, None,
                             None, ws, len(ws), None) == OK
    assert lib.matpl_dp_eval(1, ctypes.byref(m), 1, 4, 100, 0, None, None, None, None, None, None,
                             None, ws, len(ws), None) == INVALID
    assert b"null" in lib.matpl_last_error()
    n = ctypes.c_int(-1)
    assert lib.matpl_profile_collect(4, None, 64, None, None, None) == INVALID
    assert lib.matpl_profile_collect(4, None, 64, None, None, ctypes.byref(n)) == INVALID
    assert lib.matpl_profile_collect(0, None, 0, None, None, ctypes.byref(n)) == OK
    assert n.value == 0


def test_md_entry_points_validate_on_the_host():
    """The batched-MD kernels refuse bad sizes, dtype codes and NULL pointers before any CUDA
    call, and an empty system is a no-op."""
    lib = _lib.load()
    OK, INVALID, DTYPE = 0, 1, 2
    assert lib.matpl_md_drift(0, 1.0, 1.0, None, None, None, None, None, None) == OK
    assert lib.matpl_md_drift(10, 1.0, 1.0, None, None, None, None, None, None) == INVALID
    assert lib.matpl_md_drift(10, 0.0, 1.0, None, None, None, None, None, None) == INVALID
    assert lib.matpl_md_skin_build(1, 0, 1, 100, 7.0, None, None, 0, *([None] * 12)) == OK
    assert lib.matpl_md_skin_build(1, 10, 1, 100, 7.0, None, None, 1, *([None] * 12)) == INVALID
    assert lib.matpl_md_skin_build(1, 10, 9, 100, 7.0, None, None, 1, *([None] * 12)) == INVALID
    assert lib.matpl_md_skin_filter(_lib.MATPL_F32, 0, 1, 100, 100, 6.0, *([None] * 11)) == OK
    assert lib.matpl_md_skin_filter(_lib.MATPL_F32, 10, 1, 100, 100, 6.0,
                                    *([None] * 11)) == INVALID
    assert lib.matpl_md_skin_filter(_lib.MATPL_MIXED, 10, 1, 100, 100, 6.0,
                                    *([None] * 11)) == DTYPE
    assert lib.matpl_md_kick(_lib.MATPL_F64, 1, 0, 1.0, 103.6, *([None] * 10)) == OK
    assert lib.matpl_md_kick(_lib.MATPL_F64, 1, 2, 1.0, 103.6, *([None] * 10)) == INVALID
    assert lib.matpl_md_kick(_lib.MATPL_F64, 2, 2, 1.0, 103.6, *([None] * 10)) == INVALID
    assert lib.matpl_md_kick(7, 1, 2, 1.0, 103.6, *([None] * 10)) == DTYPE


def test_fit_dual_validates_on_the_host():
    """The training fitting kernel refuses bad dtypes, NULL pointers and a short workspace before
    any CUDA call; no rows is a no-op."""
    lib = _lib.load()
    OK, INVALID, DTYPE, WORKSPACE = 0, 1, 2, 3
    call = lambda dt, n, ws, nb: lib.matpl_dp_fit_dual(dt, n, *([None] * 8), ws, nb, None)  # noqa: E731
    assert call(_lib.MATPL_F32, 0, None, 0) == OK
    assert call(_lib.MATPL_MIXED, 10, None, 0) == DTYPE
    assert call(_lib.MATPL_F32, -1, None, 0) == INVALID
    assert call(_lib.MATPL_F32, 10, None, 0) == INVALID            # NULL arrays
    assert lib.matpl_dp_fit_dual_workspace_bytes(_lib.MATPL_F32, 1000) >= 13 * 1000 * 50 * 4
    assert lib.matpl_dp_fit_dual_workspace_bytes(_lib.MATPL_F64, 1000) >= 13 * 1000 * 50 * 8
    assert lib.matpl_dp_fit_dual_workspace_bytes(_lib.MATPL_MIXED, 1000) == 0


def test_nep_skin_entry_points_validate_on_the_host():
    """The NEP skin-list update and filter refuse bad sizes, NULL pointers and a short workspace
    before any CUDA call; an empty system is a no-op."""
    lib = _lib.load()
    OK, INVALID, UNSUPPORTED = 0, 1, 5
    upd = lambda nf, n, r, skin, cap, ws=None, nb=0: lib.matpl_nep_skin_update(  # noqa: E731
        nf, n, *([None] * 5), r, skin, cap, *([None] * 8), ws, nb, None)
    assert upd(1, 0, 7.0, 1.0, 100) == OK
    assert upd(0, 10, 7.0, 1.0, 100) == INVALID
    assert upd(1, 10, 0.0, 1.0, 100) == INVALID
    assert upd(1, 10, 7.0, -1.0, 100) == INVALID
    assert upd(1, 10, 7.0, 1.0, 0) == INVALID
    assert upd(1, 10, 7.0, 1.0, 6000) == UNSUPPORTED
    assert upd(1, 10, 7.0, 1.0, 100) == INVALID            # NULL arrays
    filt = lambda n, rr, ra, cap: lib.matpl_nep_skin_filter(  # noqa: E731
        1, n, None, rr, ra, 80, 30, 1, cap, *([None] * 10), 0, None)
    assert filt(0, 6.0, 4.0, 100) == OK
    assert filt(10, 6.0, 0.0, 100) == INVALID
    assert filt(10, 6.0, 4.0, 0) == INVALID
    assert filt(10, 6.0, 4.0, 100) == INVALID               # NULL arrays
    comp = lambda n, rr, cap: lib.matpl_nep_skin_filter_compact(  # noqa: E731
        n, rr, 4.0, 80, 30, cap, *([None] * 12))
    assert comp(0, 6.0, 100) == OK
    assert comp(10, 0.0, 100) == INVALID
    assert comp(10, 6.0, 0) == INVALID
    assert comp(10, 6.0, 100) == INVALID                   # NULL arrays


def test_noalloc_neighbor_search_refuses_oversize_requests_on_the_host():
    """The allocation-free search has a fixed scratch array; a request that needs more is
    refused before any CUDA call (200,000 atoms need far more than its 4 MiB)."""
    lib = _lib.load()
    rct = (ctypes.c_double * 1)(6.0)
    st = lib.matpl_neighbor_build_noalloc(1, 200000, 1, 100, 6.0, rct, None, None, None,
                                          _lib.MATPL_F64, None, None, None, None, None)
    assert st == 3   # MATPL_ERR_WORKSPACE
    assert b"4 MiB" in lib.matpl_last_error()


def test_workspace_queries():
    lib = _lib.load()
    assert lib.matpl_neighbor_workspace_bytes(1, 32000) > 32000 * 24
    assert lib.matpl_dp_workspace_bytes(0, 1, 32000) >= 32000 * 100 * 4 * 2
    assert lib.matpl_dp_param_count(2) == 4 * dp.EMB_SIZE + 2 * dp.FIT_SIZE


def test_pack_params_layout_roundtrip():
    cfg = P.DPConfig(atom_type=[3, 14])
    prm = P.init_params(cfg, seed=1)
    flat = dp.pack_params(cfg, prm)
    assert flat.numel() == _lib.load().matpl_dp_param_count(2)
    k = 3  # embedding net (1, 1)
    base = k * dp.EMB_SIZE
    w1 = flat[base + 2 * dp.E: base + 2 * dp.E + dp.E * dp.E].reshape(dp.E, dp.E)
    assert torch.equal(w1, prm["embedding_net.3.layers.1.weight"])
    # no resnet_dt in the embedding -> packed as ones
    dt1 = flat[base + 3 * dp.E + dp.E * dp.E: base + 4 * dp.E + dp.E * dp.E]
    assert torch.equal(dt1, torch.ones(dp.E, dtype=torch.float64))
    fb = 4 * dp.EMB_SIZE + dp.FIT_SIZE   # fitting net 1
    W0 = prm["fitting_net.1.layers.0.weight"]
    assert torch.equal(flat[fb:fb + dp.DIN * dp.F].reshape(dp.DIN, dp.F), W0)
    assert torch.equal(flat[fb + dp.FIT_W0T: fb + dp.FIT_W1T].reshape(dp.F, dp.DIN), W0.t())
    assert flat[fb + dp.FIT_B3] == prm["fitting_net.1.layers.3.bias"].reshape(-1)[0]


def test_per_type_stats_rejects_untiled():
    cfg = P.DPConfig(atom_type=[29])
    a = torch.zeros(1, cfg.nslots * 4)
    a[0, 4] = 1.0
    with pytest.raises(_lib.MatplError):
        dp.per_type_stats(a, 1)


def _c_layout(tmp_path, struct, fields):
    """sizeof and offsetof of a header struct as the C compiler lays it out."""
    src = tmp_path / f"{struct}.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "matpl_gb300.h"',
             'int main(void) {', f'    printf("%zu\\n", sizeof({struct}));']
    lines += [f'    printf("%zu\\n", offsetof({struct}, {f}));' for f in fields]
    lines += ['    return 0;', '}']
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / struct
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(REPO, "include"), str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    return int(out[0]), [int(v) for v in out[1:]]


@pytest.mark.parametrize("struct,mirror", [("matpl_dp_model", _lib.MatplDpModel),
                                           ("matpl_nep_model", _lib.MatplNepModel)])
def test_ctypes_structs_match_the_header_layout(tmp_path, struct, mirror):
    """The ctypes mirrors have the C compiler's size and field offsets (an offset that drifts
    would hand the kernels a wrong device pointer)."""
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    names = [f[0] for f in mirror._fields_]
    size, offs = _c_layout(tmp_path, struct, names)
    assert ctypes.sizeof(mirror) == size
    for n, off in zip(names, offs):
        assert getattr(mirror, n).offset == off, n


def test_error_codes_and_dtype_codes_match_the_header():
    txt = open(os.path.join(REPO, "include", "matpl_gb300.h")).read()
    kerr = dict(re.findall(r"#define MATPL_KERR_([A-Z_]+) (\d+)", txt))
    assert kerr and all(getattr(_lib, "KERR_" + k) == int(v) for k, v in kerr.items())
    dt = dict(re.findall(r"\bMATPL_(F32|F64|MIXED|MIXED_FAST|MIXED_TANHF) = (\d+)", txt))
    assert dt == {"F32": "0", "F64": "1", "MIXED": "2", "MIXED_FAST": "3", "MIXED_TANHF": "4"}


def _header_prototypes():
    txt = open(os.path.join(REPO, "include", "matpl_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    protos = {}
    for ret, name, params in re.findall(r"([A-Za-z_][\w \*]*?)\b(matpl_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;",
                                        txt):
        ps = [p.strip() for p in params.split(",") if p.strip()]
        protos[name] = [] if ps == ["void"] else ps
    return protos


def _c_class(decl):
    if "*" in decl:
        return "ptr"
    if "double" in decl:
        return "f64"
    if "long long" in decl:
        return "i64"
    if "size_t" in decl:
        return "size"
    return "i32"


def _ctypes_class(t):
    if t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, "contents"):
        return "ptr"
    return {ctypes.c_double: "f64", ctypes.c_longlong: "i64", ctypes.c_size_t: "size",
            ctypes.c_int: "i32"}.get(t, repr(t))


def test_ctypes_signatures_match_the_header_prototypes():
    """Every ctypes signature has the header's parameter count and, per parameter, the same
    class (pointer, int, long long, size_t, double)."""
    protos = _header_prototypes()
    assert set(protos) == set(header_functions())
    for name, params in protos.items():
        _, argtypes = _lib.SIGNATURES[name]
        assert len(argtypes) == len(params), name
        for i, (p, t) in enumerate(zip(params, argtypes)):
            assert _c_class(p) == _ctypes_class(t), f"{name} parameter {i}: {p!r} vs {t!r}"


def test_empty_slot_entry_points_validate_on_the_host():
    """The training empty-slot kernels refuse bad dtypes, present lists, NULL pointers and a
    short workspace before any CUDA call."""
    lib = _lib.load()
    INVALID, DTYPE, WORKSPACE = 1, 2, 3
    nb = lib.matpl_dp_pad_workspace_bytes(2)
    assert nb >= 2 * 2 * 100 * 8 and nb % 16 == 0
    assert lib.matpl_dp_pad_workspace_bytes(0) == 0 and lib.matpl_dp_pad_workspace_bytes(9) == 0
    m = _lib.MatplDpModel()
    m.ntypes, m.m, m.npresent, m.present[0], m.present[1] = 2, 100, 2, 0, 1
    p = ctypes.c_void_p(16)            # never dereferenced: every call below fails first
    m.params = m.davg = m.dstd = 16
    fwd = lambda dt, md, ws, nb, a=p: lib.matpl_dp_pad_forward(  # noqa: E731
        dt, ctypes.byref(md), 1, 10, 200, p, p, p, a, p, ws, nb, None)
    bwd = lambda dt, md, ws, nb, g=p: lib.matpl_dp_pad_backward(  # noqa: E731
        dt, ctypes.byref(md), 1, 10, 200, p, p, p, g, ws, nb, None)
    for call in (fwd, bwd):
        assert call(_lib.MATPL_MIXED, m, p, nb) == DTYPE
        assert call(_lib.MATPL_F32, m, p, nb - 1) == WORKSPACE
        assert call(_lib.MATPL_F32, m, None, nb) == WORKSPACE
    assert fwd(_lib.MATPL_F32, m, p, nb, a=None) == INVALID
    assert bwd(_lib.MATPL_F64, m, p, nb, g=None) == INVALID
    m.present[1] = 2
    assert fwd(_lib.MATPL_F32, m, p, nb) == INVALID and b"present" in lib.matpl_last_error()
    m.present[1], m.npresent = 1, 9
    assert bwd(_lib.MATPL_F32, m, p, nb) == INVALID
