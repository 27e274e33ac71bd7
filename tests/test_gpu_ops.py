"""calculateForce / calculateVirial drop-ins and their backward, and the environment matrix,
against the oracle restatements of the reference ops."""
import numpy as np
import pytest
import torch

from matpl_gb300 import ops
from oracle import dp_oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


def op_inputs(c, dtype, seed=0, nghost=0):
    g = torch.Generator().manual_seed(seed)
    ln = torch.tensor(c.list_neigh)
    idr = torch.tensor(c.image_dr, dtype=dtype)
    B, N, S = ln.shape
    Ri, Ri_d = dp_oracle.env_matrix(c.cfg, idr, torch.tensor(c.types), c.davg, c.dstd)
    dE = torch.randn(B, N, 4 * S, generator=g, dtype=torch.float64).to(dtype)
    ln0 = (ln - 1).to(torch.int32)
    if nghost:
        # route some neighbors to ghost rows N..N+nghost-1 (LAMMPS layout)
        gsel = (ln0 >= 0) & (torch.rand(ln0.shape, generator=g) < 0.2)
        ln0 = torch.where(gsel, N + (ln0 % nghost), ln0)
    return ln0, dE, Ri_d.reshape(B, N, 4 * S, 3).to(dtype), idr[..., 1:].contiguous()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("nghost", [0, 7])
def test_force_virial_ops_match_oracle(golden_case, dtype, nghost):
    c = golden_case("lisi600_f64")
    ln0, dE, Rd, Rij = op_inputs(c, dtype, nghost=nghost)
    B, N, S = ln0.shape
    Fc = -(dE.reshape(B, N, 1, 4 * S) @ Rd).squeeze(-2)
    F_ref, V_ref, AV_ref = dp_oracle.force_virial_ops(ln0, dE, Rd, Rij, Fc, nghost)
    d = lambda t: t.to(DEV)
    F = ops.calculateForce(d(ln0.unsqueeze(2)), d(dE.reshape(B, N, 1, 4 * S)), d(Rd), d(Fc),
                           torch.tensor(nghost))[0]
    V, AV = ops.calculateVirial(d(ln0.unsqueeze(2)), d(dE.reshape(B, N, 1, 4 * S)), d(Rij), d(Rd),
                                torch.tensor(nghost))
    tol = 1e-11 if dtype == torch.float64 else 2e-4
    fs = F_ref.abs().max().item()
    np.testing.assert_allclose(F.cpu().numpy(), F_ref.numpy(), rtol=0, atol=tol * fs)
    vs = V_ref.abs().max().item()
    np.testing.assert_allclose(V.cpu().numpy(), V_ref.numpy(), rtol=0, atol=tol * vs * 10)
    np.testing.assert_allclose(AV.cpu().numpy(), AV_ref.numpy(), rtol=0,
                               atol=tol * AV_ref.abs().max().item())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_force_virial_backward_match_oracle(golden_case, dtype):
    c = golden_case("cu108_f64")
    ln0, dE, Rd, Rij = op_inputs(c, dtype, seed=3)
    B, N, S = ln0.shape
    g = torch.Generator().manual_seed(5)
    gF = torch.randn(B, N, 3, generator=g, dtype=torch.float64).to(dtype)
    gV = torch.randn(B, 9, generator=g, dtype=torch.float64).to(dtype)
    ref_f, ref_v = dp_oracle.force_virial_grads(ln0, Rd, Rij, gF, gV)
    dEg = dE.reshape(B, N, 1, 4 * S).to(DEV).requires_grad_()
    Fc = torch.zeros(B, N, 3, dtype=dtype, device=DEV)
    F = ops.calculateForce(ln0.unsqueeze(2).to(DEV), dEg, Rd.to(DEV), Fc, 0)[0]
    (gf,) = torch.autograd.grad(F, dEg, gF.to(DEV))
    V = ops.calculateVirial(ln0.unsqueeze(2).to(DEV), dEg, Rij.to(DEV), Rd.to(DEV), 0)[0]
    (gv,) = torch.autograd.grad(V, dEg, gV.to(DEV))
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    np.testing.assert_allclose(gf.reshape(B, N, 4 * S).cpu().numpy(), ref_f.numpy(), rtol=0,
                               atol=tol * ref_f.abs().max().item())
    np.testing.assert_allclose(gv.reshape(B, N, 4 * S).cpu().numpy(), ref_v.numpy(), rtol=0,
                               atol=tol * ref_v.abs().max().item())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_env_mat_matches_oracle(golden_case, dtype):
    for name in ["cu108_f64", "hfo2_jit"]:
        c = golden_case(name)
        idr = torch.tensor(c.image_dr, dtype=dtype)
        Ri_ref, Rid_ref = dp_oracle.env_matrix(c.cfg, idr, torch.tensor(c.types), c.davg, c.dstd)
        Ri, Rid = ops.env_mat(idr.to(DEV), torch.tensor(c.types).to(DEV), c.davg, c.dstd,
                              c.cfg.Rmin, c.cfg.Rmax)
        tol = 1e-12 if dtype == torch.float64 else 1e-5
        np.testing.assert_allclose(Ri.cpu().numpy(), Ri_ref.numpy(), rtol=tol,
                                   atol=tol * Ri_ref.abs().max().item())
        np.testing.assert_allclose(Rid.cpu().numpy(), Rid_ref.numpy(), rtol=tol,
                                   atol=tol * Rid_ref.abs().max().item())


def test_ops_reject_cpu_tensors(golden_case):
    c = golden_case("cu108_f64")
    ln0, dE, Rd, Rij = op_inputs(c, torch.float64)
    from matpl_gb300 import _lib
    with pytest.raises(_lib.MatplError):
        ops.calculateForce(ln0, dE, Rd, torch.zeros(1, 108, 3, dtype=torch.float64), 0)
