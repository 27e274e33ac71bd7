"""Force-loss training on a ragged batch: configurations of uneven atom count and
composition (Hf:O 1:2, 3 % cell strain, density 0.07) concatenated by ``data.ragged_batch``
into one image, the loss E-MSE over the configurations' energies + F-MSE.

Gradients of every parameter against second-order autograd through the FP64 oracle on the
same concatenated configurations (each configuration's list from the oracle search on its own
cell, indices shifted by its first atom), a finite-difference check, and the graphed step
against the eager one."""
import numpy as np
import pytest
import torch

from matpl_gb300 import data, params as P, structures, train
from oracle import dp_oracle, neigh

pytestmark = pytest.mark.gpu
DEV = "cuda"
COUNTS = (32, 45, 61, 33, 48, 40)


def make_configs(counts=COUNTS, seed=100):
    cfg = P.DPConfig(atom_type=[72, 8], maxNeighborNum=100)
    sts = [structures.random_packed(n, 0.07, [72, 8], [1 / 3, 2 / 3], seed=seed + k, strain=0.03)
           for k, n in enumerate(counts)]
    return cfg, sts


def oracle_lists(cfg, sts):
    lns, idrs, start = [], [], 0
    for st in sts:
        ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, 100, 6.0, [6.0, 6.0])
        lns.append(np.where(ln > 0, ln + start, 0))
        idrs.append(idr)
        start += st.natoms
    types = np.concatenate([st.types for st in sts]).astype(np.int32)
    cfg_of = np.concatenate([np.full(st.natoms, c) for c, st in enumerate(sts)])
    return np.concatenate(lns, 1), np.concatenate(idrs, 1), types, cfg_of


def oracle_energies(cfg, prm, davg, dstd, ln, idr, types, cfg_of, C, create_graph=False):
    out = dp_oracle.dp_eval(cfg, prm, torch.tensor(davg), torch.tensor(dstd), torch.tensor(ln),
                            torch.tensor(types), torch.tensor(cfg.atom_type), torch.tensor(idr), 0,
                            create_graph=create_graph)
    E = torch.zeros(C, dtype=torch.float64).index_add(0, torch.tensor(cfg_of),
                                                      out["Ei_atom"].reshape(-1))
    return E, out["Force"]


@pytest.fixture(scope="module")
def case():
    cfg, sts = make_configs()
    ln, idr, types, cfg_of = oracle_lists(cfg, sts)
    davg, dstd = P.calc_stat(cfg, ln, idr, types)
    prm = P.init_params(cfg, 5)
    teacher = P.init_params(cfg, 99)
    C = len(sts)
    E_t, F_t = oracle_energies(cfg, teacher, davg, dstd, ln, idr, types, cfg_of, C)
    g = torch.Generator().manual_seed(3)
    E_lab = E_t.detach() + 0.01 * torch.randn(C, generator=g, dtype=torch.float64)
    F_lab = F_t.detach() + 0.01 * torch.randn(F_t.shape, generator=g, dtype=torch.float64)
    # oracle gradients: second-order autograd through the FP64 restatement
    p = {k: v.clone().requires_grad_() for k, v in prm.items()}
    E, F = oracle_energies(cfg, p, davg, dstd, ln, idr, types, cfg_of, C, create_graph=True)
    loss = torch.nn.functional.mse_loss(E, E_lab) + torch.nn.functional.mse_loss(F, F_lab)
    names = sorted(p)
    gr = torch.autograd.grad(loss, [p[k] for k in names])
    batch = data.ragged_batch(cfg, sts, device=DEV,
                              energies=E_lab.numpy(),
                              forces=[f.numpy() for f in torch.split(F_lab[0], list(COUNTS))])
    return dict(cfg=cfg, sts=sts, ln=ln, idr=idr, davg=davg, dstd=dstd, prm=prm, batch=batch,
                loss=loss.item(), grads=dict(zip(names, gr)))


def test_ragged_collate_equals_the_oracle_lists(case):
    b = case["batch"]
    assert np.array_equal(b["list_neigh"].cpu().numpy(), case["ln"])
    assert np.array_equal(b["ImageDR"].cpu().numpy().view(np.uint64), case["idr"].view(np.uint64))
    assert b["natoms"].tolist() == list(COUNTS)
    assert b["config_of_atom"].shape[0] == sum(COUNTS)


@pytest.mark.parametrize("dtype,eval_precision,tol", [(torch.float64, None, 1e-8),
                                                      (torch.float32, None, 2e-3),
                                                      (torch.float32, "mixed", 2e-3)])
def test_ragged_fused_gradients_match_oracle(case, dtype, eval_precision, tol):
    model = train.DPTrainModel(case["cfg"], case["prm"], case["davg"], case["dstd"], dtype=dtype,
                               device=DEV)
    b = dict(case["batch"])
    b["ImageDR"] = b["ImageDR"].to(dtype)
    loss, _, _ = train.FusedTrainer(model, eval_precision).loss_and_backward(b)
    assert abs(loss - case["loss"]) <= (1e-10 if dtype == torch.float64 else 1e-4) * case["loss"]
    worst, where = 0.0, None
    for k, gr in case["grads"].items():
        got = model.param(k).grad.detach().double().cpu()
        err = (got - gr).abs().max().item() / (gr.abs().max().item() + 1e-30)
        if err > worst:
            worst, where = err, k
    print(f"[accuracy] ragged fused training gradients {dtype} (evaluation "
          f"{eval_precision or 'same'}): worst relative error {worst:.2e} ({where})")
    assert worst < tol, (worst, where)


def test_ragged_plain_step_matches_oracle(case):
    model = train.DPTrainModel(case["cfg"], case["prm"], case["davg"], case["dstd"],
                               dtype=torch.float64, device=DEV)
    loss, _, _ = train.loss_fn(model, case["batch"])
    loss.backward()
    assert abs(loss.item() - case["loss"]) <= 1e-10 * case["loss"]
    for k, gr in case["grads"].items():
        got = model.param(k).grad.detach().cpu()
        assert (got - gr).abs().max().item() <= 1e-8 * (gr.abs().max().item() + 1e-30), k


def test_ragged_fused_gradient_finite_difference(case):
    model = train.DPTrainModel(case["cfg"], case["prm"], case["davg"], case["dstd"],
                               dtype=torch.float64, device=DEV)
    tr = train.FusedTrainer(model)
    b = case["batch"]
    for name, q in (("embedding_net.1.layers.2.weight", 11), ("fitting_net.0.layers.1.bias", 3)):
        p = model.param(name)
        flat = p.detach().view(-1)
        h = 1e-6
        vals = []
        for sgn in (1, -1):
            with torch.no_grad():
                flat[q] += sgn * h
            vals.append(tr.loss_and_backward(b)[0])
            with torch.no_grad():
                flat[q] -= sgn * h
        fd = (vals[0] - vals[1]) / (2 * h)
        model.zero_grad(set_to_none=True)
        tr.loss_and_backward(b)
        got = model.param(name).grad.view(-1)[q].item()
        assert abs(fd - got) <= 1e-5 * max(1.0, abs(fd)), (name, fd, got)


def test_ragged_graphed_step_matches_eager(case):
    cfg, b = case["cfg"], case["batch"]
    m1 = train.DPTrainModel(cfg, case["prm"], case["davg"], case["dstd"], dtype=torch.float64,
                            device=DEV)
    m2 = train.DPTrainModel(cfg, case["prm"], case["davg"], case["dstd"], dtype=torch.float64,
                            device=DEV)
    o1 = torch.optim.SGD(m1.parameters(), lr=1e-5)
    o2 = torch.optim.SGD(m2.parameters(), lr=1e-5)
    t1 = train.FusedTrainer(m1)
    g2 = train.GraphedTrainer(train.FusedTrainer(m2), o2, warmup=2)
    for _ in range(2):
        t1.step([b], o1)
    for _ in range(3):
        l1 = t1.step([b], o1)
        l2 = float(g2.step(b))
        assert abs(l1 - l2) <= 1e-10 * abs(l1)
    for k in m1.names:
        assert torch.allclose(m1.param(k), m2.param(k), rtol=1e-10, atol=1e-12), k


def test_ragged_graphed_step_with_tensor_core_evaluation(case):
    """The FP32 step whose evaluation runs on the tensor cores: graphed = eager, and its
    gradients within 1e-4 (relative to each parameter's largest) of the FP32-evaluation step."""
    cfg, b = case["cfg"], dict(case["batch"])
    b["ImageDR"] = b["ImageDR"].float()
    m0 = train.DPTrainModel(cfg, case["prm"], case["davg"], case["dstd"], dtype=torch.float32,
                            device=DEV)
    mx = train.DPTrainModel(cfg, case["prm"], case["davg"], case["dstd"], dtype=torch.float32,
                            device=DEV)
    train.FusedTrainer(m0).loss_and_backward(b)
    train.FusedTrainer(mx, "mixed").loss_and_backward(b)
    for k in m0.names:
        g0, gx = m0.param(k).grad, mx.param(k).grad
        assert float((gx - g0).abs().max()) <= 1e-4 * float(g0.abs().max()) + 1e-12, k
    m1 = train.DPTrainModel(cfg, case["prm"], case["davg"], case["dstd"], dtype=torch.float32,
                            device=DEV)
    m2 = train.DPTrainModel(cfg, case["prm"], case["davg"], case["dstd"], dtype=torch.float32,
                            device=DEV)
    o1 = torch.optim.SGD(m1.parameters(), lr=1e-5)
    o2 = torch.optim.SGD(m2.parameters(), lr=1e-5)
    t1 = train.FusedTrainer(m1, "mixed")
    g2 = train.GraphedTrainer(train.FusedTrainer(m2, "mixed"), o2, warmup=2)
    for _ in range(2):                 # the graphed trainer's two warm-up steps
        t1.step([b], o1)
    for _ in range(3):
        l1 = t1.step([b], o1)
        l2 = float(g2.step(b))
        # FP32 force sums by atomics: the two runs differ in summation order only
        assert abs(l1 - l2) <= 1e-5 * abs(l1)
