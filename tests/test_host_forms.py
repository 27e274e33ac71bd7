"""Host-side reformulations of the training and variant paths, checked against the reference's
structure on the CPU (no GPU): the all-element NEP fitting product, the per-image sums, the
batched DP empty-slot term and the type-embedding model folded into per-pair nets."""
import types

import torch

from matpl_gb300 import nep as NP, params as P
from matpl_gb300.nep_train import NEPTrain, _image_sum
from matpl_gb300.train import DPTrainModel, FusedTrainer
from matpl_gb300.typedp import TypeDP, dp_params, init_type_params


def test_nep_all_element_fitting_equals_per_element_nets():
    cfg = NP.NepConfig(atom_type=[8, 72, 14, 3])
    m = NEPTrain(cfg, NP.init_params(cfg, 5), dtype=torch.float64, device="cpu")
    g = torch.Generator().manual_seed(3)
    feats = torch.randn(500, cfg.feature_nums, generator=g, dtype=torch.float64,
                        requires_grad=True)
    tm = torch.randint(0, 4, (500,), generator=g)
    Ei = m.calculate_Ei(tm, feats)
    ref = torch.zeros(500, dtype=torch.float64)
    for t, net in enumerate(m.fitting_net):
        idx = (tm == t).nonzero().flatten()
        ref = ref.index_put((idx,), net(feats[idx]).squeeze(-1))
    torch.testing.assert_close(Ei, ref, rtol=1e-13, atol=1e-13)
    ps = [feats] + list(m.fitting_net.parameters())
    g1 = torch.autograd.grad((Ei ** 2).sum(), ps, create_graph=True)
    g2 = torch.autograd.grad((ref ** 2).sum(), ps, create_graph=True)
    for a, b in zip(g1, g2):
        torch.testing.assert_close(a, b, rtol=1e-12, atol=1e-12)
    v = torch.randn(feats.shape, generator=g, dtype=torch.float64)
    h1 = torch.autograd.grad((g1[0] * v).sum(), ps[1:])
    h2 = torch.autograd.grad((g2[0] * v).sum(), ps[1:])
    for a, b in zip(h1, h2):
        torch.testing.assert_close(a, b, rtol=1e-11, atol=1e-11)


def test_image_sums_equal_and_unequal_frames():
    x = torch.randn(12, 3, 3, dtype=torch.float64)
    for counts in ((4, 4, 4), (5, 3, 4), (12,)):
        ref = torch.stack([c.sum(0) for c in x.split(list(counts))])
        torch.testing.assert_close(_image_sum(x, counts), ref)


def test_dp_batched_empty_slot_term_equals_pairwise_sum():
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=50)
    model = DPTrainModel(cfg, P.init_params(cfg, 5), torch.rand(2, 400), torch.rand(2, 400) + 0.5,
                         dtype=torch.float64, device="cpu")
    g = torch.Generator().manual_seed(4)
    B, N, m = 2, 30, 50
    ln = (torch.rand(B, N, 2 * m, generator=g) > 0.6).to(torch.int32)
    tm = torch.randint(0, 2, (N,), generator=g)
    davg4 = torch.rand(2, 4, generator=g, dtype=torch.float64)
    dstd4 = torch.rand(2, 4, generator=g, dtype=torch.float64) + 0.5
    fake = types.SimpleNamespace(model=model, davg4=davg4, dstd4=dstd4, _tm_long=tm)
    out = FusedTrainer._pad_term(fake, ln, [0, 1])
    occ = (ln > 0).reshape(B, N, 2, m).sum(-1)
    ref = torch.zeros(B, N, 4, 25, dtype=torch.float64)
    for ti in (0, 1):
        rp = (0.0 - davg4[ti]) / dstd4[ti]
        sel = (tm == ti).to(torch.float64).reshape(1, N, 1, 1)
        for tj in (0, 1):
            G = model._emb(ti * 2 + tj, rp[0:1].reshape(1, 1))[0]
            nemp = (m - occ[:, :, tj]).to(torch.float64).reshape(B, N, 1, 1)
            ref = ref + sel * nemp * (rp.reshape(4, 1) * G.reshape(1, 25))
    torch.testing.assert_close(out, ref, rtol=1e-13, atol=1e-12)
    ps = list(model.parameters())
    g1 = torch.autograd.grad(out.pow(2).sum(), ps, allow_unused=True)
    g2 = torch.autograd.grad(ref.pow(2).sum(), ps, allow_unused=True)
    for a, b in zip(g1, g2):
        assert (a is None) == (b is None)
        if a is not None:
            torch.testing.assert_close(a, b, rtol=1e-12, atol=1e-9)


def test_type_embedding_folds_into_per_pair_nets():
    cfg = P.DPConfig(atom_type=[72, 8], maxNeighborNum=100)
    prm = init_type_params(cfg, 3, 7)
    vec = {72: [0.1, 0.2, 0.3], 8: [0.4, -0.1, 0.05]}
    d = dp_params(cfg, prm, vec)
    m = TypeDP(cfg, prm, torch.zeros(2, 800), torch.ones(2, 800), vec, device="cpu")
    s = torch.randn(9, 1, dtype=torch.float64)
    for k in range(4):
        q = f"embedding_net.{k}.layers."
        x = torch.tanh(s @ d[q + "0.weight"] + d[q + "0.bias"])
        for layer in (1, 2):
            h = torch.tanh(x @ d[q + f"{layer}.weight"] + d[q + f"{layer}.bias"])
            dt = d.get(q + f"{layer}.resnet_dt")
            x = (h * dt if dt is not None else h) + x
        torch.testing.assert_close(x, m._emb(k, s), rtol=1e-14, atol=1e-14)
