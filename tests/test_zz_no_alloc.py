"""The allocation-free neighbor search (matpl_neighbor_build_noalloc), called through the C ABI.

It exists for hosts that cannot give the library device memory (an MD engine's force callback
that owns all device memory, a C / Fortran host without an allocator); its scratch is a fixed
array inside the library.  This file sorts last so that a failure here cannot hide others.
The test checks two calls in a row (a larger structure, then a smaller one, so the second call
runs on scratch left over from the first) against the workspace entry point, bit for bit.  The
refusal of an oversize request needs no GPU and is checked with the host-side validation tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from matpl_gb300 import _lib, structures

pytestmark = pytest.mark.gpu
DEV = "cuda"


def run(lib, st, ntypes, m, noalloc):
    N = len(st.types)
    S = ntypes * m
    tm = torch.tensor(st.types, dtype=torch.int32, device=DEV)
    lat = torch.tensor(st.lattice, dtype=torch.float64, device=DEV).reshape(1, 3, 3).contiguous()
    pos = torch.tensor(st.frac, dtype=torch.float64, device=DEV).reshape(1, N, 3).contiguous()
    ln = torch.full((1, N, S), -7, dtype=torch.int32, device=DEV)
    idr = torch.full((1, N, S, 4), float("nan"), dtype=torch.float64, device=DEV)
    cnt = torch.full((1, N, ntypes), -7, dtype=torch.int32, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    rct = (ctypes.c_double * ntypes)(*([6.0] * ntypes))
    stream = torch.cuda.current_stream().cuda_stream
    if noalloc:
        st_code = lib.matpl_neighbor_build_noalloc(1, N, ntypes, m, 6.0, rct, tm.data_ptr(),
                                                   lat.data_ptr(), pos.data_ptr(), _lib.MATPL_F64,
                                                   ln.data_ptr(), idr.data_ptr(), cnt.data_ptr(),
                                                   err.data_ptr(), stream)
    else:
        nbytes = lib.matpl_neighbor_workspace_bytes(1, N)
        ws = torch.empty(nbytes, dtype=torch.uint8, device=DEV)
        st_code = lib.matpl_neighbor_build(1, N, ntypes, m, 6.0, rct, tm.data_ptr(), lat.data_ptr(),
                                           pos.data_ptr(), _lib.MATPL_F64, ln.data_ptr(),
                                           idr.data_ptr(), cnt.data_ptr(), err.data_ptr(),
                                           ws.data_ptr(), nbytes, stream)
    assert st_code == 0, lib.matpl_last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return ln.cpu().numpy(), idr.cpu().numpy(), cnt.cpu().numpy()


def test_noalloc_matches_workspace_entry_point_twice():
    lib = _lib.load()
    big = structures.random_packed(20000, 0.05, [3, 14], [0.5, 0.5], seed=77)
    small = structures.random_packed(3000, 0.07, [72, 8], [1 / 3, 2 / 3], seed=78, strain=0.03)
    for st in (big, small):          # second call reuses the first call's scratch contents
        ref = run(lib, st, 2, 150, noalloc=False)
        got = run(lib, st, 2, 150, noalloc=True)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
        assert (ref[0] > 0).sum() > 0
