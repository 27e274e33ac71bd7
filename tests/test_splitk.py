"""Split-K products (matpl_gb300.splitk) on the host: the batched partial products equal the
plain product, and their gradients to second order equal torch's."""
import torch

from matpl_gb300 import splitk


def test_split_product_equals_plain_product():
    g = torch.Generator().manual_seed(1)
    for K in (100, 8192, 20000, 20011):                  # below, at and above the split size
        a = torch.randn(K, 35, generator=g, dtype=torch.float64).t()   # transposed view
        b = torch.randn(K, 40, generator=g, dtype=torch.float64)
        torch.testing.assert_close(splitk.mm(a, b), a @ b, rtol=1e-12, atol=1e-10)


def test_gradients_to_second_order():
    g = torch.Generator().manual_seed(2)
    x = torch.randn(9000, 12, generator=g, dtype=torch.float64, requires_grad=True)
    w = torch.randn(12, 7, generator=g, dtype=torch.float64, requires_grad=True)
    b = torch.randn(1, 7, generator=g, dtype=torch.float64, requires_grad=True)

    def f(mm, add):
        return torch.tanh(add(mm(x, w), b)).pow(2).sum()
    ours = f(splitk.mm, splitk.add_row)
    ref = f(lambda p, q: p @ q, lambda z, c: z + c)
    torch.testing.assert_close(ours, ref, rtol=1e-12, atol=0)
    g1 = torch.autograd.grad(ours, [x, w, b], create_graph=True)
    g2 = torch.autograd.grad(ref, [x, w, b], create_graph=True)
    for p, q in zip(g1, g2):
        torch.testing.assert_close(p, q, rtol=1e-11, atol=1e-9)
    v = torch.randn(x.shape, generator=g, dtype=torch.float64)
    h1 = torch.autograd.grad((g1[0] * v).sum(), [w, b])
    h2 = torch.autograd.grad((g2[0] * v).sum(), [w, b])
    for p, q in zip(h1, h2):
        torch.testing.assert_close(p, q, rtol=1e-10, atol=1e-8)
