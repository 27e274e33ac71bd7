"""Pin the oracle's NEP training derivatives against golden vectors made by MatPL's own NEP code
(the CPU branch of nep_net.NEP under autograd): the first and second backward of the descriptor
(what calculateNepFeat / calculateNepMbFeat and their Grad functions return) and the training
gradient of an energy + force + virial loss through NEP.forward."""
import numpy as np
import pytest
import torch

from oracle import nep_oracle as NO

CASES = [("nep_q4_tri2", "nep_train_q4_tri2"), ("nep_hfo_l4", "nep_train_hfo_l4")]


def seeded(seed, shape):
    return np.random.default_rng(int(seed)).standard_normal(shape)


def load(name):
    from tests.conftest import load_golden
    return load_golden(name)


def close(a, b, tol):
    a = a.detach().numpy() if isinstance(a, torch.Tensor) else a
    np.testing.assert_allclose(a, b, rtol=0, atol=tol * max(1.0, np.abs(b).max()))


@pytest.mark.parametrize("case,train", CASES)
def test_oracle_descriptor_derivatives(nep_case, case, train):
    c = nep_case(case)
    t = load(train)
    cfg = c.cfg
    N, F = c.NL_r.shape[0], cfg.feature_nums
    tm = torch.tensor(c.g["type_map"])
    c2 = c.params["c_param_2"].clone().requires_grad_()
    c3 = c.params["c_param_3"].clone().requires_grad_() if cfg.l_max[0] > 0 else None
    Rr = torch.tensor(c.Ri_r).requires_grad_()
    Ra = torch.tensor(c.Ri_a).requires_grad_()
    q = [NO.features_2b(cfg, c2, tm, torch.tensor(c.NL_r), Rr)]
    if c3 is not None:
        q.append(NO.features_mb(cfg, c3, tm, torch.tensor(c.NL_a), Ra))
    q = torch.cat(q, -1)
    G = torch.tensor(seeded(t["seed_G"], (N, F))).requires_grad_()
    params = [c2] + ([c3] if c3 is not None else [])
    first = torch.autograd.grad((q * G).sum(), params + [Rr, Ra], create_graph=True,
                                allow_unused=True)
    close(first[0], t["first_c2"], 1e-12)
    close(first[len(params)], t["first_Rr"], 1e-12)
    gRa = first[len(params) + 1]
    if c3 is not None:
        close(first[1], t["first_c3"], 1e-12)
        close(gRa, t["first_Ra"], 1e-12)
    Hr = torch.tensor(seeded(t["seed_Hr"], tuple(c.Ri_r.shape)))
    Ha = torch.tensor(seeded(t["seed_Ha"], tuple(c.Ri_a.shape)))
    L2 = (first[len(params)] * Hr).sum() + ((gRa * Ha).sum() if gRa is not None else 0)
    second = torch.autograd.grad(L2, [G] + params, allow_unused=True)
    close(second[0], t["second_G"], 1e-12)
    close(second[1], t["second_c2"], 1e-12)
    if c3 is not None:
        close(second[2], t["second_c3"], 1e-12)


@pytest.mark.parametrize("case,train", CASES)
def test_oracle_training_gradient(nep_case, case, train):
    c = nep_case(case)
    t = load(train)
    N = c.NL_r.shape[0]
    B = len(c.g["num_atom"])
    gE = seeded(t["seed_gE"], (B,))
    gF = seeded(t["seed_gF"], (N, 3))
    gV = seeded(t["seed_gV"], (B, 9))
    g = NO.train_grads(c.cfg, c.params, c.g["num_atom"], c.g["type_map"], c.NL_r, c.Ri_r,
                       c.NL_a, c.Ri_a, gE, gF, gV)
    keys = [k[6:] for k in t if k.startswith("train:")]
    assert set(keys) == set(g.keys())
    for k in keys:
        close(g[k], t["train:" + k], 1e-11)
