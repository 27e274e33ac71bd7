"""Matrix products whose contraction runs over the atoms (the weight and bias gradients of the
per-atom fitting nets in the training steps) as split-K batched products, differentiable to any
order.  A single GEMM of shape [F, N_atoms] x [N_atoms, H] gets a handful of output tiles and
runs on a few SMs; S partial products of ~256 atoms in one batched launch plus their sum use
the whole GPU.  Used by ``nep_train.NEPTrain`` and ``train.FusedTrainer``.
"""
import torch


def _mm_impl(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """a [M, K] @ b [K, N].  A long contraction onto few outputs (the weight and bias gradients
    of the fitting net, K = atoms) goes as S partial products of about 256 atoms in one
    batched launch plus their sum: the work spreads over the SMs instead of the handful of
    output tiles a single GEMM of that shape gets."""
    M, K = a.shape
    N = b.shape[1]
    if K < 8192 or M * N > 256 * 256:
        return a @ b
    S = min(128, K // 256)
    c = K // S
    K0 = S * c
    out = torch.bmm(a[:, :K0].reshape(M, S, c).transpose(0, 1), b[:K0].reshape(S, c, N)).sum(0)
    if K0 < K:
        out = out + a[:, K0:] @ b[K0:]
    return out


class _MM(torch.autograd.Function):
    """Matrix product through ``_mm_impl`` in the forward and every order of backward."""

    @staticmethod
    def forward(ctx, a, b):
        ctx.save_for_backward(a, b)
        return _mm_impl(a, b)

    @staticmethod
    def backward(ctx, g):
        a, b = ctx.saved_tensors
        ga = _MM.apply(g, b.t()) if ctx.needs_input_grad[0] else None
        gb = _MM.apply(a.t(), g) if ctx.needs_input_grad[1] else None
        return ga, gb


_ones_rows = {}


def _ones_row(n, dev, dt):
    key = (n, dev, dt)
    t = _ones_rows.get(key)
    if t is None:
        if len(_ones_rows) > 16:
            _ones_rows.clear()
        t = _ones_rows[key] = torch.ones(1, n, dtype=dt, device=dev)
    return t


class _AddRow(torch.autograd.Function):
    """z [N, F] + b [F]; the gradient of b, a sum over the N rows, as ones[1, N] @ g through
    ``_MM`` (differentiable again)."""

    @staticmethod
    def forward(ctx, z, b):
        ctx.n = z.shape[0]
        return z + b

    @staticmethod
    def backward(ctx, g):
        gb = None
        if ctx.needs_input_grad[1]:
            gb = _MM.apply(_ones_row(ctx.n, g.device, g.dtype), g).reshape(-1)
        return g, gb


def mm(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """a @ b (2-D), differentiable, long contractions split."""
    return _MM.apply(a, b)


def add_row(z: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """z [N, F] + b [F] (or [1, F]), the gradient of b through ``mm``."""
    return _AddRow.apply(z, b.reshape(-1))
