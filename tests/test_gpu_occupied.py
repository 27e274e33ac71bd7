"""The occupied-slot path of the fused step (matpl_neighbor_build_occupied +
matpl_dp_eval_occupied) against the zero-filled drop-in path, and the bounded-wait exit of the
tensor-core kernels.

* The occupied-slot search writes exactly the occupied slots of the drop-in list (same
  indices, same ImageDR bits) and the same block lengths; empty slots are left untouched.
* The evaluation on the occupied-slot list, with every empty slot poisoned, equals the
  evaluation on the zero-filled list in every precision form.
* A completion wait that gives up (the wait bound shrunk to a single check) surfaces as
  MATPL_KERR_TIMEOUT from the Python API, and the next evaluation on the same context is
  correct again.
"""
import numpy as np
import pytest
import torch

from matpl_gb300 import _lib, dp, ops, params as P, structures

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _box(n=3000, seed=31):
    st = structures.random_packed(n, 0.05, [3, 14], [0.5, 0.5], seed=seed)
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150)
    return st, cfg


def _lists(st, out_dtype, occupied):
    return ops.find_neighbore(torch.tensor(st.types), torch.tensor(st.frac, device=DEV),
                              torch.tensor(st.lattice), 2, 150, 6.0, 6.0, out_dtype=out_dtype,
                              with_counts=True, occupied_only=occupied)


@pytest.mark.parametrize("out_dtype", [torch.float64, torch.float32])
def test_occupied_search_writes_the_occupied_slots_only(out_dtype):
    st, _ = _box()
    ln, idr, cnt = _lists(st, out_dtype, False)
    # poison the outputs first: the occupied-slot search must leave the empty slots alone
    N, S = ln.shape[1], ln.shape[2]
    lnp = torch.full_like(ln, -7)
    idrp = torch.full_like(idr, float("nan"))
    cntp = torch.empty_like(cnt)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    lib = _lib.load()
    ws = ops.workspace(torch.device(DEV), lib.matpl_neighbor_workspace_bytes(1, N), "neighbor")
    import ctypes
    rct = (ctypes.c_double * 2)(6.0, 6.0)
    lat = torch.tensor(st.lattice, device=DEV).reshape(1, 3, 3).contiguous()
    pos = torch.tensor(st.frac, device=DEV).reshape(1, N, 3).contiguous()
    tm = torch.tensor(st.types, dtype=torch.int32, device=DEV)
    code = {torch.float64: _lib.MATPL_F64, torch.float32: _lib.MATPL_F32}[out_dtype]
    _lib.check(lib.matpl_neighbor_build_occupied(
        1, N, 2, 150, 6.0, rct, tm.data_ptr(), lat.data_ptr(), pos.data_ptr(), code,
        lnp.data_ptr(), idrp.data_ptr(), cntp.data_ptr(), err.data_ptr(), ws.data_ptr(),
        ws.numel(), torch.cuda.current_stream().cuda_stream), "occupied")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(cntp, cnt)
    k = torch.arange(S, device=DEV) % 150
    blk = torch.arange(S, device=DEV) // 150
    occ = k.view(1, 1, S) < torch.gather(cnt, 2, blk.view(1, 1, S).expand(1, N, S))
    assert torch.equal(occ, ln > 0)
    assert torch.equal(lnp[occ], ln[occ])
    assert bool((lnp[~occ] == -7).all())
    a = idrp[occ].cpu().numpy()
    b = idr[occ].cpu().numpy()
    view = np.uint64 if out_dtype == torch.float64 else np.uint32
    assert np.array_equal(a.view(view), b.view(view))
    assert bool(torch.isnan(idrp[~occ]).all())


@pytest.mark.parametrize("precision", ["float64", "float32", "mixed", "mixed_tanhf", "mixed_fast"])
def test_occupied_evaluation_equals_the_drop_in_path(precision):
    st, cfg = _box(2400, seed=32)
    prm = P.init_params(cfg, 5)
    ln64, idr64, _ = _lists(st, torch.float64, False)
    davg, dstd = P.calc_stat(cfg, ln64.cpu().numpy(), idr64.cpu().numpy(), st.types)
    m = dp.DP(cfg, prm, davg, dstd, precision=precision, device=DEV)
    ln, idr, cnt = _lists(st, m.dtype, False)
    present = m.present_types(cfg.atom_type)
    tm = torch.tensor(st.types, dtype=torch.int32, device=DEV)
    ref = m.evaluate(ln, tm, present, idr, 0)
    ref = {k: v.clone() for k, v in ref.items()}
    empty = ln == 0
    ln_p = ln.masked_fill(empty, 123456)                 # never read
    idr_p = idr.masked_fill(empty.unsqueeze(-1), float("nan"))
    got = m.evaluate(ln_p, tm, present, idr_p, 0, num_neigh=cnt)
    torch.cuda.synchronize()
    tol = 1e-12 if precision == "float64" else 1e-5
    for k in ("Etot", "Ei_atom", "Force", "Virial"):
        scale = ref[k].abs().max().item()
        err = (got[k] - ref[k]).abs().max().item()
        assert np.isfinite(err) and err <= tol * max(scale, 1.0), (k, err, scale)


def test_bounded_wait_gives_up_cleanly_and_the_context_stays_usable():
    st, cfg = _box(1200, seed=33)
    prm = P.init_params(cfg, 6)
    ln64, idr64, _ = _lists(st, torch.float64, False)
    davg, dstd = P.calc_stat(cfg, ln64.cpu().numpy(), idr64.cpu().numpy(), st.types)
    m = dp.DP(cfg, prm, davg, dstd, precision="mixed", device=DEV)
    ln, idr, cnt = _lists(st, torch.float32, True)
    present = m.present_types(cfg.atom_type)
    tm = torch.tensor(st.types, dtype=torch.int32, device=DEV)
    good = m.evaluate(ln, tm, present, idr, 0, num_neigh=cnt)
    good = {k: v.clone() for k, v in good.items()}
    lib = _lib.load()
    try:
        _lib.check(lib.matpl_dp_set_wait_limit(1), "matpl_dp_set_wait_limit")
        with pytest.raises(_lib.MatplError, match="MATPL_KERR_TIMEOUT"):
            m.evaluate(ln, tm, present, idr, 0, num_neigh=cnt)
    finally:
        _lib.check(lib.matpl_dp_set_wait_limit(0), "matpl_dp_set_wait_limit")
    again = m.evaluate(ln, tm, present, idr, 0, num_neigh=cnt)
    torch.cuda.synchronize()
    for k in ("Etot", "Force", "Virial"):
        scale = good[k].abs().max().item()
        assert (again[k] - good[k]).abs().max().item() <= 1e-5 * max(scale, 1.0), k
