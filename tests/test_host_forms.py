"""Host-side reformulations of the training and variant paths, checked against the reference's
structure on the CPU (no GPU): the all-element NEP fitting product, the per-image sums and the
type-embedding model folded into per-pair nets."""
import torch

from matpl_gb300 import nep as NP, params as P
from matpl_gb300.nep_train import NEPTrain, _image_sum
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
