"""torch.ops.CalcOps_cuda (libCalcOps_bind.so) on the GPU, called the way MatPL's models call
the reference's operators:

* calculateForce / calculateVirial with the arguments of the DP CUDA branch
  (src/model/dp_dp.py:461-469: list_neigh [B,N,1,S] int32 0-based, dE [B,N,1,4S],
  Ri_d [B,N,4S,3], the centre term, nghost as a 0-d int64 tensor on the device) fed the
  reference's own dE of the golden case: the reference's forces and virial to 1e-10; the
  backward against the oracle's transpose;
* calculateCompress = this package's operator (and its backward);
* calculate_neighbor / calculate_maxneigh = the reference CPU operator's lists (fixture), bit
  for bit; calculateNepForce / calculateNepVirial = the oracle scatter.
"""
import numpy as np
import pytest
import torch

from matpl_gb300 import build, ops
from oracle import dp_oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def calcops():
    build.build()
    torch.ops.load_library(build.OPS_LIB)
    return torch.ops.CalcOps_cuda


def test_dp_force_virial_as_the_dp_cuda_branch_calls_them(golden_case, calcops):
    c = golden_case("cu108_f64")
    g = c.g
    idr = torch.tensor(c.image_dr)
    Ri, Ri_d = dp_oracle.env_matrix(c.cfg, idr, torch.tensor(c.types), c.davg, c.dstd)
    B, N, S = c.list_neigh.shape
    Rd = Ri_d.reshape(B, N, 4 * S, 3).to(DEV)
    dE = torch.tensor(g["dE"]).reshape(B, N, 1, 4 * S).to(DEV)      # the reference's own dE
    Force = -1 * torch.matmul(dE, Rd).squeeze(-2)
    ImageDR = idr[..., 1:].clone().to(DEV)
    nghost_tensor = torch.tensor(0, device=DEV, dtype=torch.int64)
    list_neigh = (torch.unsqueeze(torch.tensor(c.list_neigh, device=DEV), 2) - 1).type(torch.int)
    F = calcops.calculateForce(list_neigh, dE, Rd, Force, nghost_tensor)[0]
    V = calcops.calculateVirial(list_neigh, dE, ImageDR, Rd, nghost_tensor)[0]
    np.testing.assert_allclose(F.cpu().numpy(), g["Force"], rtol=0,
                               atol=1e-10 * np.abs(g["Force"]).max())
    np.testing.assert_allclose(V.cpu().numpy(), g["Virial"], rtol=0,
                               atol=1e-10 * np.abs(g["Virial"]).max())


@pytest.mark.parametrize("nghost", [0, 5])
def test_dp_ops_backward_match_the_oracle(golden_case, calcops, nghost):
    c = golden_case("lisi600_f64")
    idr = torch.tensor(c.image_dr)
    _, Ri_d = dp_oracle.env_matrix(c.cfg, idr, torch.tensor(c.types), c.davg, c.dstd)
    B, N, S = c.list_neigh.shape
    gen = torch.Generator().manual_seed(1)
    dE = torch.randn(B, N, 4 * S, generator=gen, dtype=torch.float64)
    ln0 = torch.tensor(c.list_neigh).to(torch.int32) - 1
    if nghost:
        sel = (ln0 >= 0) & (torch.rand(ln0.shape, generator=gen) < 0.2)
        ln0 = torch.where(sel, N + (ln0 % nghost), ln0)
    Rd = Ri_d.reshape(B, N, 4 * S, 3)
    Rij = idr[..., 1:].contiguous()
    gF = torch.randn(B, N + nghost, 3, generator=gen, dtype=torch.float64)
    gV = torch.randn(B, 9, generator=gen, dtype=torch.float64)
    Fc = -(dE.reshape(B, N, 1, 4 * S) @ Rd).squeeze(-2)
    F_ref, V_ref, _ = dp_oracle.force_virial_ops(ln0, dE, Rd, Rij, Fc, nghost)
    dEg = dE.reshape(B, N, 1, 4 * S).to(DEV).requires_grad_()
    nt = torch.tensor(nghost, device=DEV)
    F = calcops.calculateForce(ln0.unsqueeze(2).to(DEV), dEg, Rd.to(DEV), Fc.to(DEV), nt)[0]
    V = calcops.calculateVirial(ln0.unsqueeze(2).to(DEV), dEg, Rij.to(DEV), Rd.to(DEV), nt)[0]
    np.testing.assert_allclose(F.detach().cpu().numpy(), F_ref.numpy(), rtol=0,
                               atol=1e-11 * F_ref.abs().max().item())
    np.testing.assert_allclose(V.detach().cpu().numpy(), V_ref.numpy(), rtol=0,
                               atol=1e-10 * V_ref.abs().max().item())
    (gd,) = torch.autograd.grad((F * gF.to(DEV)).sum() + (V * gV.to(DEV)).sum(), [dEg])
    # the same through this package's autograd drop-ins
    dE2 = dE.reshape(B, N, 1, 4 * S).to(DEV).requires_grad_()
    F2 = ops.calculateForce(ln0.unsqueeze(2).to(DEV), dE2, Rd.to(DEV), Fc.to(DEV), nghost)[0]
    V2 = ops.calculateVirial(ln0.unsqueeze(2).to(DEV), dE2, Rij.to(DEV), Rd.to(DEV), nghost)[0]
    (gd2,) = torch.autograd.grad((F2 * gF.to(DEV)).sum() + (V2 * gV.to(DEV)).sum(), [dE2])
    assert torch.allclose(gd, gd2, rtol=1e-12, atol=1e-12)


def test_compress_matches_the_package_operator(calcops):
    gen = torch.Generator().manual_seed(2)
    f2 = torch.rand(500, 1, generator=gen, dtype=torch.float64).to(DEV).requires_grad_()
    coef = torch.randn(500, 25, 6, generator=gen, dtype=torch.float64).to(DEV)
    G = calcops.calculateCompress(f2, coef)[0]
    G2 = ops.calculateCompress(f2, coef)[0]
    assert torch.equal(G, G2)
    (a,) = torch.autograd.grad(G.sum(), [f2])
    (b,) = torch.autograd.grad(G2.sum(), [f2])
    assert torch.equal(a, b)


def test_nep_neighbor_ops_equal_the_reference_fixture(nep_case, calcops):
    c = nep_case("nep_q4_240")
    fr = c.frames
    t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=DEV)  # noqa: E731
    args = (t(fr.num_atom.reshape(-1, 1), torch.int64), t(fr.type_map, torch.int64),
            torch.arange(len(c.cfg.atom_type), device=DEV), t(fr.box, torch.float64),
            t(fr.box_orig, torch.float64), t(fr.num_cell, torch.int64),
            t(fr.position, torch.float64))
    g = c.g
    got = calcops.calculate_neighbor(*args, c.cfg.cutoff[0], c.cfg.cutoff[1], int(g["max_r"]),
                                     int(g["max_a"]), True)
    ref = (c.NN_r, c.NN_a, c.NL_r, c.NL_a, c.Ri_r, c.Ri_a)
    for a, b in zip(got, ref):
        assert np.array_equal(a.cpu().numpy(), b)
    cnt = calcops.calculate_maxneigh(args[0], args[3], args[4], args[5], args[6],
                                     c.cfg.cutoff[0], c.cfg.cutoff[1], len(c.cfg.atom_type),
                                     args[1], False)
    assert torch.equal(cnt[0], got[0]) and torch.equal(cnt[1], got[1])


def test_nep_force_virial_ops_match_the_oracle(nep_case, calcops):
    c = nep_case("nep_q4_240")
    N, NN = c.NL_r.shape
    gen = torch.Generator().manual_seed(4)
    dE = torch.randn(N, 4 * NN, generator=gen, dtype=torch.float64)
    Ri_d = torch.randn(N, 4 * NN, 3, generator=gen, dtype=torch.float64)
    Rij = torch.tensor(c.Ri_r[..., 1:])
    nl = torch.tensor(c.NL_r)
    Fc = torch.randn(N, 3, generator=gen, dtype=torch.float64)
    F_ref, _, AV_ref = dp_oracle.force_virial_ops(nl.reshape(1, N, NN), dE.reshape(1, N, 4 * NN),
                                                  Ri_d.reshape(1, N, 4 * NN, 3),
                                                  Rij.reshape(1, N, NN, 3), Fc.reshape(1, N, 3), 0)
    F = calcops.calculateNepForce(nl.to(DEV), dE.to(DEV), Ri_d.to(DEV), Fc.to(DEV))[0]
    np.testing.assert_allclose(F.cpu().numpy(), F_ref[0].numpy(), rtol=0,
                               atol=1e-11 * F_ref.abs().max().item())
    counts = torch.tensor(c.frames.num_atom).reshape(-1)
    V, AV = calcops.calculateNepVirial(nl.to(DEV), dE.to(DEV), Rij.to(DEV), Ri_d.to(DEV), counts)
    np.testing.assert_allclose(AV.cpu().numpy(), AV_ref[0].numpy(), rtol=0,
                               atol=1e-11 * AV_ref.abs().max().item())
    img = torch.repeat_interleave(torch.arange(counts.numel()), counts)
    V_ref = torch.zeros(counts.numel(), 9, dtype=torch.float64).index_add_(0, img, AV_ref[0])
    np.testing.assert_allclose(V.cpu().numpy(), V_ref.numpy(), rtol=0,
                               atol=1e-11 * V_ref.abs().max().item())
