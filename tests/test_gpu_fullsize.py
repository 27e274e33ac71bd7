"""The headline configurations at full size against the oracle.

* DP: the 32,000-atom Li/Si box (0.05 atoms/A^3, seed 2024, m = 150 per type).  The GPU
  neighbor list and ImageDR equal the C restatement of ``NeighConst.f90:14-149`` bit for bit;
  the FP64 energy, per-atom energies, forces and virial are within 1e-10 relative of the
  torch-FP64 restatement of ``dp_dp_script.DP`` (evaluated in chunks of centre atoms); the
  plain FP32 and the tcgen05 mixed forms stay within the 1e-4 eV/A force bar of that oracle.
* NEP: the 100,000-atom, four-element box (0.06 atoms/A^3): both neighbor lists (indices and
  the (r, x, y, z) rows) equal the C restatement of the reference CPU operator
  (``cpu_calculate_nepneighbor.cpp:105-203``) bit for bit.
"""
import os
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from matpl_gb300 import dp, nep as NP, ops, params as P, structures
from oracle import dp_oracle, neigh, nep_oracle as NO

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def lisi32k():
    torch.set_num_threads(os.cpu_count() or 1)
    st = structures.random_packed(32000, 0.05, [3, 14], [0.5, 0.5], seed=2024)
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150)
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, 150, 6.0, [6.0, 6.0])
    sub = slice(0, 2000)
    davg, dstd = P.calc_stat(cfg, ln[:, sub], idr[:, sub], st.types[sub])
    prm = P.init_params(cfg, 11)
    ref = dp_oracle.dp_eval_chunked(cfg, prm, torch.tensor(davg), torch.tensor(dstd),
                                    torch.tensor(ln), torch.tensor(st.types),
                                    torch.tensor(cfg.atom_type), torch.tensor(idr), chunk=4000)
    return SimpleNamespace(st=st, cfg=cfg, ln=ln, idr=idr, davg=davg, dstd=dstd, prm=prm,
                           ref={k: v.detach() for k, v in ref.items()})


def _gpu_lists(c, out_dtype=torch.float64):
    return ops.find_neighbore(torch.tensor(c.st.types), torch.tensor(c.st.frac, device=DEV),
                              torch.tensor(c.st.lattice), 2, 150, 6.0, 6.0, out_dtype=out_dtype)


def test_32k_neighbor_list_bit_exact_vs_oracle(lisi32k):
    c = lisi32k
    ln, idr = _gpu_lists(c)
    assert int((ln > 0).sum()) == int((c.ln > 0).sum()) > 1_400_000
    assert np.array_equal(ln.cpu().numpy(), c.ln)
    assert np.array_equal(idr.cpu().numpy().view(np.uint64), c.idr.view(np.uint64))
    # the FP32 output is the FP64 list rounded to nearest
    ln32, idr32 = _gpu_lists(c, torch.float32)
    assert np.array_equal(ln32.cpu().numpy(), c.ln)
    assert np.array_equal(idr32.cpu().numpy(), c.idr.astype(np.float32))


def _evaluate(c, precision):
    m = dp.DP(c.cfg, c.prm, c.davg, c.dstd, precision=precision, device=DEV)
    ln, idr = _gpu_lists(c, m.dtype)
    present = m.present_types(c.cfg.atom_type)
    out = m.evaluate(ln, torch.tensor(c.st.types, dtype=torch.int32, device=DEV), present, idr, 0)
    torch.cuda.synchronize()
    assert int(m.err.item()) == 0
    return {k: v.double().cpu() for k, v in out.items()}


def test_32k_fp64_matches_oracle(lisi32k):
    """E / Ei / F / V of the FP64 GPU path within 1e-10 relative of the oracle."""
    c, ref = lisi32k, lisi32k.ref
    out = _evaluate(c, "float64")
    tol = 1e-10
    assert abs(out["Etot"].item() - ref["Etot"].item()) <= tol * abs(ref["Etot"].item())
    emax = ref["Ei_atom"].abs().max().item()
    assert (out["Ei_atom"] - ref["Ei_atom"]).abs().max().item() <= tol * emax
    fmax = ref["Force"].abs().max().item()
    assert (out["Force"] - ref["Force"]).abs().max().item() <= 10 * tol * fmax
    vmax = ref["Virial"].abs().max().item()
    assert (out["Virial"] - ref["Virial"]).abs().max().item() <= 10 * tol * vmax


@pytest.mark.parametrize("precision", ["float32", "mixed", "mixed_tanhf"])
def test_32k_reduced_precision_forms_within_force_bar_of_oracle(lisi32k, precision):
    """Force RMSE <= 1e-4 eV/A against the FP64 oracle; energy and virial errors printed."""
    c, ref = lisi32k, lisi32k.ref
    out = _evaluate(c, precision)
    rmse = (out["Force"] - ref["Force"]).pow(2).mean().sqrt().item()
    e_err = abs(out["Etot"].item() - ref["Etot"].item()) / 32000
    v_err = (out["Virial"] - ref["Virial"]).abs().max().item() / ref["Virial"].abs().max().item()
    print(f"[accuracy vs oracle] {precision} 32k Li/Si: force RMSE {rmse:.3e} eV/A, "
          f"energy {e_err:.3e} eV/atom, virial {v_err:.3e} relative")
    assert rmse <= 1e-4, rmse
    assert e_err < 2e-4, e_err


def test_nep_100k_lists_bit_exact_vs_oracle():
    torch.set_num_threads(os.cpu_count() or 1)
    cfg = NP.NepConfig(atom_type=[3, 14, 8, 72])
    st = structures.random_packed(100_000, 0.06, [3, 14, 8, 72], [0.25] * 4, seed=4)
    fr = NP.frames_from_structures([st], cfg.cutoff[0])
    t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=DEV)  # noqa: E731
    mr, ma = 90, 36
    got = ops.calculate_neighbor(t(fr.num_atom.reshape(-1, 1), torch.int64),
                                 t(fr.type_map, torch.int64), torch.arange(4, device=DEV),
                                 t(fr.box, torch.float64), t(fr.box_orig, torch.float64),
                                 t(fr.num_cell, torch.int64), t(fr.position, torch.float64),
                                 cfg.cutoff[0], cfg.cutoff[1], mr, ma, True)
    got = [g.cpu().numpy() for g in got]
    ref = NO.neighbor(fr, cfg.cutoff[0], cfg.cutoff[1], mr, ma)
    assert int(ref[0].sum()) > 5_000_000
    for k in range(4):                       # NN_r, NN_a, NL_r, NL_a
        assert np.array_equal(got[k], ref[k]), k
    for k in (4, 5):                         # Ri_r, Ri_a bit for bit
        assert np.array_equal(got[k].view(np.uint64), ref[k].view(np.uint64)), k
