"""calculateCompress drop-in (tabulated embedding) and its backward against the oracle."""
import numpy as np
import pytest
import torch

from matpl_gb300 import ops
from oracle import dp_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("coe_num", [4, 6])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_compress_forward_backward(coe_num, dtype):
    g = torch.Generator().manual_seed(coe_num)
    ns, nodes = 4099, 25
    f2 = (torch.rand(ns, 1, generator=g, dtype=torch.float64) * 0.02).to(dtype)
    coef = torch.randn(ns, nodes, coe_num, generator=g, dtype=torch.float64).to(dtype)
    G_ref, dG_ref = dp_oracle.compress_oracle(f2, coef)
    fd = f2.cuda().requires_grad_()
    G = ops.calculateCompress(fd, coef.cuda())[0]
    gG = torch.randn(ns, nodes, generator=g, dtype=torch.float64).to(dtype)
    (gf,) = torch.autograd.grad(G, fd, gG.cuda())
    tol = 1e-12 if dtype == torch.float64 else 2e-6
    np.testing.assert_allclose(G.detach().cpu().double().numpy(), G_ref.numpy(), rtol=0,
                               atol=tol * G_ref.abs().max().item())
    ref_gf = (gG.double() * dG_ref).sum(-1, keepdim=True)
    np.testing.assert_allclose(gf.cpu().double().numpy(), ref_gf.numpy(), rtol=0,
                               atol=tol * 10 * ref_gf.abs().max().item())


def test_compress_rejects_other_orders():
    from matpl_gb300 import _lib
    with pytest.raises(_lib.MatplError):
        ops.calculateCompress(torch.zeros(3, 1, device="cuda"), torch.zeros(3, 25, 5, device="cuda"))


def test_compress_empty():
    G = ops.calculateCompress(torch.zeros(0, 1, device="cuda"), torch.zeros(0, 25, 4, device="cuda"))[0]
    assert G.shape == (0, 25)
