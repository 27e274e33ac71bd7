"""NEP training operators on the GPU against MatPL's own NEP code (golden fixtures from the CPU
branch of nep_net.NEP under autograd) and the oracle: descriptor forward / backward / second
backward (calculateNepFeat, calculateNepMbFeat), and the training gradient of an energy + force
+ virial loss through NEPTrain (NEP.forward's CUDA branch on this library's operators)."""
import numpy as np
import pytest
import torch

from matpl_gb300 import nep as NP, nep_ops, structures
from matpl_gb300.nep_train import NEPTrain
from oracle import nep_oracle as NO

pytestmark = pytest.mark.gpu
DEV = "cuda"
CASES = [("nep_q4_tri2", "nep_train_q4_tri2"), ("nep_hfo_l4", "nep_train_hfo_l4")]


def seeded(seed, shape):
    return np.random.default_rng(int(seed)).standard_normal(shape)


def load(name):
    from tests.conftest import load_golden
    return load_golden(name)


def close(a, b, tol):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    np.testing.assert_allclose(a, b, rtol=0, atol=tol * max(1.0, np.abs(b).max()))


def dev(a, dt=None):
    t = torch.as_tensor(np.ascontiguousarray(a) if isinstance(a, np.ndarray) else a)
    return t.to(device=DEV, dtype=dt if dt is not None else t.dtype)


def gpu_feats(c, dt, c2, c3, Rr, Ra):
    cfg = c.cfg
    N = c.NL_r.shape[0]
    tm = dev(c.g["type_map"])
    q = [nep_ops.calculateNepFeat(c2, Rr, dev(c.NL_r), tm, torch.zeros(N, cfg.nr, dtype=dt,
                                                                    device=DEV),
                                  cfg.cutoff[0], cfg.multi_feat_num)[0]]
    if c3 is not None:
        q.append(nep_ops.calculateNepMbFeat(c3, Ra, dev(c.NL_a), tm,
                                            torch.zeros(N, cfg.multi_feat_num, dtype=dt,
                                                        device=DEV),
                                            cfg.nr, *cfg.l_max, cfg.cutoff[1])[0])
    return torch.cat(q, -1)


@pytest.mark.parametrize("case", ["nep_q4_240", "nep_q4_tri2", "nep_hfo_l4"])
def test_feat_forward_matches_reference(nep_case, case):
    c = nep_case(case)
    c2 = dev(c.params["c_param_2"])
    c3 = dev(c.params["c_param_3"]) if c.cfg.l_max[0] > 0 else None
    q = gpu_feats(c, torch.float64, c2, c3, dev(c.Ri_r), dev(c.Ri_a))
    close(q, c.g["feats"], 1e-12)


@pytest.mark.parametrize("case,train", CASES)
def test_feat_first_and_second_backward(nep_case, case, train):
    c = nep_case(case)
    t = load(train)
    cfg = c.cfg
    N, F = c.NL_r.shape[0], cfg.feature_nums
    c2 = dev(c.params["c_param_2"]).requires_grad_()
    c3 = dev(c.params["c_param_3"]).requires_grad_() if cfg.l_max[0] > 0 else None
    Rr = dev(c.Ri_r).requires_grad_()
    Ra = dev(c.Ri_a).requires_grad_()
    q = gpu_feats(c, torch.float64, c2, c3, Rr, Ra)
    G = dev(seeded(t["seed_G"], (N, F))).requires_grad_()
    params = [c2] + ([c3] if c3 is not None else [])
    first = torch.autograd.grad((q * G).sum(), params + [Rr, Ra], create_graph=True,
                                allow_unused=True)
    close(first[0], t["first_c2"], 1e-11)
    close(first[len(params)], t["first_Rr"], 1e-11)
    gRa = first[len(params) + 1]
    if c3 is not None:
        close(first[1], t["first_c3"], 1e-11)
        close(gRa, t["first_Ra"], 1e-11)
    Hr = dev(seeded(t["seed_Hr"], tuple(c.Ri_r.shape)))
    Ha = dev(seeded(t["seed_Ha"], tuple(c.Ri_a.shape)))
    L2 = (first[len(params)] * Hr).sum() + ((gRa * Ha).sum() if gRa is not None else 0)
    second = torch.autograd.grad(L2, [G] + params, allow_unused=True)
    close(second[0], t["second_G"], 1e-11)
    close(second[1], t["second_c2"], 1e-11)
    if c3 is not None:
        close(second[2], t["second_c3"], 1e-11)


def nep_train_model(c, dt=torch.float64):
    return NEPTrain(c.cfg, c.params, dtype=dt, device=DEV)


def run_step(model, c, gE, gF, gV, dt=torch.float64):
    model.zero_grad(set_to_none=True)
    Etot, Ei, F, _, V = model(dev(c.NN_r), dev(c.NL_r), dev(c.Ri_r, dt), dev(c.NN_a),
                              dev(c.NL_a), dev(c.Ri_a, dt), dev(c.g["num_atom"]),
                              dev(c.g["type_map"]))
    L = (dev(gE, dt) * Etot.reshape(-1)).sum() + (dev(gF, dt) * F).sum() + (dev(gV, dt) * V).sum()
    L.backward()
    return Etot, F, V, {k: v.grad for k, v in model.named_parameters()}


@pytest.mark.parametrize("case,train", CASES)
def test_training_gradient_matches_reference(nep_case, case, train):
    c = nep_case(case)
    t = load(train)
    N = c.NL_r.shape[0]
    B = len(c.g["num_atom"])
    gE, gF, gV = (seeded(t["seed_gE"], (B,)), seeded(t["seed_gF"], (N, 3)),
                  seeded(t["seed_gV"], (B, 9)))
    Etot, F, V, grads = run_step(nep_train_model(c), c, gE, gF, gV)
    close(Etot.reshape(-1), t["train_Etot"].reshape(-1), 1e-12)
    close(F, t["train_Force"], 1e-11)
    close(V, t["train_Virial"], 1e-11)
    keys = [k[6:] for k in t if k.startswith("train:")]
    assert set(keys) == set(grads)
    for k in keys:
        close(grads[k], t["train:" + k], 1e-10)


def test_training_gradient_fp32_and_larger_box():
    """A 1,200-atom four-element box: FP64 gradients = the oracle's second-order autograd,
    FP32 within 1e-4 of them (relative to the largest entry)."""
    cfg = NP.NepConfig(atom_type=[3, 14, 8, 72])
    st = structures.random_packed(1200, 0.06, [3, 14, 8, 72], [0.25] * 4, seed=77)
    fr = NP.frames_from_structures([st], cfg.cutoff[0])
    NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = NO.neighbor(fr, cfg.cutoff[0], cfg.cutoff[1], 120, 40)

    class C:
        pass
    c = C()
    c.cfg = cfg
    c.params = NP.init_params(cfg, 9, energy_shift=-3.0)
    c.params["q_scaler"] = torch.full((cfg.feature_nums,), 0.5, dtype=torch.float64)
    c.NN_r, c.NN_a, c.NL_r, c.NL_a, c.Ri_r, c.Ri_a = NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a
    c.g = {"num_atom": fr.num_atom, "type_map": fr.type_map}
    N = NL_r.shape[0]
    rng = np.random.default_rng(5)
    gE, gF, gV = rng.standard_normal(1), rng.standard_normal((N, 3)), rng.standard_normal((1, 9))
    ref = NO.train_grads(cfg, c.params, fr.num_atom, fr.type_map, NL_r, Ri_r, NL_a, Ri_a, gE, gF,
                         gV)
    _, _, _, g64 = run_step(nep_train_model(c), c, gE, gF, gV)
    for k, v in ref.items():
        close(g64[k], v.numpy(), 1e-10)
    _, _, _, g32 = run_step(nep_train_model(c, torch.float32), c, gE, gF, gV, torch.float32)
    for k, v in ref.items():
        close(g32[k].double(), v.numpy(), 1e-4)


def test_graphed_step_equals_eager_step(nep_case):
    """Two steps of the CUDA-graph trainer = two eager steps (FP64 parameters to 1e-10)."""
    from matpl_gb300 import nep_ops
    from matpl_gb300.nep_train import GraphedNepTrainer
    c = nep_case("nep_q4_tri2")
    N = c.NL_r.shape[0]
    B = len(c.g["num_atom"])
    rng = np.random.default_rng(3)
    b = {"NN_r": dev(c.NN_r), "NL_r": dev(c.NL_r), "Ri_r": dev(c.Ri_r), "NN_a": dev(c.NN_a),
         "NL_a": dev(c.NL_a), "Ri_a": dev(c.Ri_a), "type_map": dev(c.g["type_map"]),
         "num_atom": torch.tensor(c.g["num_atom"]),
         "per_atom": dev(np.asarray(c.g["num_atom"], dtype=np.float64)),
         "Etot": dev(rng.standard_normal(B)), "Force": dev(rng.standard_normal((N, 3))),
         "Virial": dev(rng.standard_normal((B, 9)))}
    m1, m2 = nep_train_model(c), nep_train_model(c)
    o1 = torch.optim.Adam(m1.parameters(), lr=1e-3, capturable=True, fused=True)
    o2 = torch.optim.Adam(m2.parameters(), lr=1e-3, capturable=True, fused=True)
    t1 = GraphedNepTrainer(m1, o1, w_v=0.1, warmup=1)
    t2 = GraphedNepTrainer(m2, o2, w_v=0.1, warmup=1)
    try:
        # the graphed trainer runs one warm-up step before capturing: match it eagerly
        for _ in range(3):
            o2.zero_grad(set_to_none=True)
            t2.loss(b).backward()
            o2.step()
        l1 = [t1.step(b) for _ in range(2)][-1]
        torch.cuda.synchronize()
        t1.check_errors()
    finally:
        nep_ops.set_check_errors(True)
    for (k, a), (_, bb) in zip(m1.named_parameters(), m2.named_parameters()):
        close(a, bb.detach().cpu().numpy(), 1e-10)
    assert torch.isfinite(l1).all()


@pytest.mark.parametrize("case", ["nep_q4_tri2", "nep_hfo_l4"])
def test_force_virial_kernel_equals_public_ops(nep_case, case):
    """nep_force_virial (Ri_d formed in the kernel) = calculate_Ri + calculateNepForce with the
    centre term + calculateNepVirial, values and the gradient in dE, for both lists."""
    from matpl_gb300.nep_train import calculate_Ri
    c = nep_case(case)
    na = np.asarray(c.g["num_atom"]).reshape(-1)
    for k, (NL, R) in enumerate(((c.NL_r, c.Ri_r), (c.NL_a, c.Ri_a))):
        N, NN = NL.shape
        R, NLd = dev(R), dev(NL)
        dE = dev(seeded(11 + k, (N, NN, 4))).requires_grad_()
        F, V = nep_ops.nep_force_virial(NLd, dE, R, na)
        Rd = calculate_Ri(R)
        f0 = -torch.matmul(dE.reshape(N, 1, -1), Rd.reshape(N, -1, 3)).squeeze(-2)
        F2 = nep_ops.calculateNepForce(NLd, dE, Rd, f0)[0]
        V2 = nep_ops.calculateNepVirial(NLd, dE, R[:, :, 1:], Rd, torch.tensor(na))[0]
        close(F, F2.detach().cpu().numpy(), 1e-13)
        close(V, V2.detach().cpu().numpy(), 1e-13)
        gF, gV = dev(seeded(21 + k, (N, 3))), dev(seeded(31 + k, (len(na), 9)))
        g1 = torch.autograd.grad((F * gF).sum() + (V * gV).sum(), dE)[0]
        g2 = torch.autograd.grad((F2 * gF).sum() + (V2 * gV).sum(), dE)[0]
        close(g1, g2.cpu().numpy(), 1e-13)
    nep_ops.check_errors()


def test_zbl_term_in_training_forward(nep_case):
    """NEPTrain with the ZBL term (outer cutoff 2.2 A, pairs in the inner and the switching
    region), FP64: E, F, V = the oracle with the kernel's float32 element factors (1e-10) and the
    reference's own values (golden, 1e-7: its float32 Z^0.23 is one ulp off for some pairs); the
    training gradient = the oracle's (the ZBL term has no parameters: it enters as constants)."""
    c = nep_case("nep_zbl")
    g = c.g
    N = c.NL_r.shape[0]
    B = len(g["num_atom"])
    rng = np.random.default_rng(8)
    gE, gF, gV = rng.standard_normal(B), rng.standard_normal((N, 3)), rng.standard_normal((B, 9))
    Etot, F, V, grads = run_step(nep_train_model(c), c, gE, gF, gV)
    ref = NO.nep_eval(c.cfg, c.params, g["num_atom"], torch.tensor(g["type_map"]),
                      torch.tensor(c.NL_r), torch.tensor(c.Ri_r), torch.tensor(c.NL_a),
                      torch.tensor(c.Ri_a), zbl_factors="rounded")
    close(Etot.reshape(-1), ref["Etot"].numpy().reshape(-1), 1e-12)
    close(F, ref["Force"].numpy(), 1e-10)
    close(V, ref["Virial"].numpy(), 1e-10)
    close(Etot.reshape(-1), g["Etot"].reshape(-1), 1e-7)     # the reference's own values
    close(F, g["Force"], 1e-7)
    ref = NO.train_grads(c.cfg, c.params, g["num_atom"], g["type_map"], c.NL_r, c.Ri_r, c.NL_a,
                         c.Ri_a, gE, gF, gV)
    for k, v in ref.items():
        close(grads[k], v.numpy(), 1e-10)
    nep_ops.check_errors()


def test_graphed_step_with_zbl_equals_eager_step(nep_case):
    """The CUDA-graph trainer with the ZBL term (FP64): two graphed steps = two eager steps."""
    from matpl_gb300.nep_train import GraphedNepTrainer
    c = nep_case("nep_zbl")
    N = c.NL_r.shape[0]
    B = len(c.g["num_atom"])
    rng = np.random.default_rng(4)
    b = {"NN_r": dev(c.NN_r), "NL_r": dev(c.NL_r), "Ri_r": dev(c.Ri_r), "NN_a": dev(c.NN_a),
         "NL_a": dev(c.NL_a), "Ri_a": dev(c.Ri_a), "type_map": dev(c.g["type_map"]),
         "num_atom": torch.tensor(c.g["num_atom"]),
         "per_atom": dev(np.asarray(c.g["num_atom"], dtype=np.float64)),
         "Etot": dev(rng.standard_normal(B)), "Force": dev(rng.standard_normal((N, 3))),
         "Virial": dev(rng.standard_normal((B, 9)))}
    m1, m2 = nep_train_model(c), nep_train_model(c)
    o1 = torch.optim.Adam(m1.parameters(), lr=1e-3, capturable=True, fused=True)
    o2 = torch.optim.Adam(m2.parameters(), lr=1e-3, capturable=True, fused=True)
    t1 = GraphedNepTrainer(m1, o1, w_v=0.1, warmup=1)
    t2 = GraphedNepTrainer(m2, o2, w_v=0.1, warmup=1)
    try:
        for _ in range(3):
            o2.zero_grad(set_to_none=True)
            t2.loss(b).backward()
            o2.step()
        l1 = [t1.step(b) for _ in range(2)][-1]
        torch.cuda.synchronize()
        t1.check_errors()
    finally:
        nep_ops.set_check_errors(True)
    for (k, a), (_, bb) in zip(m1.named_parameters(), m2.named_parameters()):
        close(a, bb.detach().cpu().numpy(), 1e-10)
    assert torch.isfinite(l1).all()
