"""Force-loss training step (dp_trainer.train on the GPU with this library's env-matrix and
force/virial kernels): parameter gradients against the FP64 oracle (second-order autograd through
MatPL's algorithm on the CPU) and against finite differences."""
import numpy as np
import pytest
import torch

from matpl_gb300 import params as P, structures, train
from oracle import dp_oracle, neigh

pytestmark = pytest.mark.gpu
DEV = "cuda"


def make_case(n=48, seed=31):
    st = structures.random_packed(n, 0.07, [72, 8], [1 / 3, 2 / 3], seed=seed, strain=0.03)
    cfg = P.DPConfig(atom_type=[72, 8], maxNeighborNum=100)
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, 100, 6.0, [6.0, 6.0])
    davg, dstd = P.calc_stat(cfg, ln, idr, st.types)
    prm = P.init_params(cfg, 5)
    teacher = P.init_params(cfg, 99)
    lab = dp_oracle.dp_eval(cfg, teacher, torch.tensor(davg), torch.tensor(dstd), torch.tensor(ln),
                            torch.tensor(st.types), torch.tensor(cfg.atom_type), torch.tensor(idr), 0)
    g = torch.Generator().manual_seed(seed)
    E_lab = lab["Etot"].detach() + 0.01 * torch.randn(1, generator=g, dtype=torch.float64)
    F_lab = lab["Force"].detach() + 0.01 * torch.randn(lab["Force"].shape, generator=g, dtype=torch.float64)
    return cfg, st, ln, idr, davg, dstd, prm, E_lab, F_lab


def oracle_grads(cfg, st, ln, idr, davg, dstd, prm, E_lab, F_lab):
    p = {k: v.clone().requires_grad_() for k, v in prm.items()}
    out = dp_oracle.dp_eval(cfg, p, torch.tensor(davg), torch.tensor(dstd), torch.tensor(ln),
                            torch.tensor(st.types), torch.tensor(cfg.atom_type), torch.tensor(idr), 0,
                            create_graph=True)
    loss = torch.nn.functional.mse_loss(out["Etot"], E_lab) + \
        torch.nn.functional.mse_loss(out["Force"], F_lab)
    names = sorted(p)
    gr = torch.autograd.grad(loss, [p[k] for k in names])
    return loss.item(), dict(zip(names, gr))


def gpu_model_and_batch(cfg, st, ln, idr, davg, dstd, prm, E_lab, F_lab):
    model = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float64, device=DEV)
    batch = {"list_neigh": torch.tensor(ln, device=DEV), "type_map": torch.tensor(st.types, device=DEV),
             "atom_type": cfg.atom_type, "ImageDR": torch.tensor(idr, device=DEV),
             "Etot": E_lab.to(DEV), "Force": F_lab.to(DEV)}
    return model, batch


def test_training_gradients_match_oracle():
    case = make_case()
    loss_ref, g_ref = oracle_grads(*case)
    model, batch = gpu_model_and_batch(*case)
    loss, _, _ = train.loss_fn(model, batch)
    loss.backward()
    assert abs(loss.item() - loss_ref) <= 1e-10 * abs(loss_ref)
    worst = 0.0
    for k, gr in g_ref.items():
        got = model.param(k).grad.detach().cpu()
        scale = gr.abs().max().item() + 1e-30
        worst = max(worst, (got - gr).abs().max().item() / scale)
    assert worst < 1e-8, worst


def test_training_gradient_finite_difference():
    case = make_case(n=36, seed=7)
    model, batch = gpu_model_and_batch(*case)
    loss, _, _ = train.loss_fn(model, batch)
    loss.backward()
    rng = np.random.default_rng(0)
    for name in ["embedding_net.1.layers.1.weight", "fitting_net.0.layers.0.weight",
                 "fitting_net.1.layers.2.resnet_dt"]:
        p = model.param(name)
        flat = p.detach().view(-1)
        for q in rng.choice(flat.numel(), 2, replace=False):
            h = 1e-6 * max(1.0, abs(flat[q].item()))
            with torch.no_grad():
                flat[q] += h
            lp = train.loss_fn(model, batch)[0].item()
            with torch.no_grad():
                flat[q] -= 2 * h
            lm = train.loss_fn(model, batch)[0].item()
            with torch.no_grad():
                flat[q] += h
            fd = (lp - lm) / (2 * h)
            an = p.grad.view(-1)[q].item()
            assert abs(fd - an) <= 1e-5 * max(1e-3, abs(an)), (name, q, fd, an)


def test_training_steps_reduce_loss():
    """Plain gradient steps with a small step size must lower the loss (the gradient is a
    descent direction)."""
    case = make_case(n=48, seed=3)
    model, batch = gpu_model_and_batch(*case)
    opt = torch.optim.SGD(model.parameters(), lr=1e-5)
    first = train.loss_fn(model, batch)[0].item()
    for _ in range(5):
        train.train_step(model, [batch], opt)
    assert train.loss_fn(model, batch)[0].item() < first


def _fused_grads(case, dtype):
    cfg, st, ln, idr, davg, dstd, prm, E_lab, F_lab = case
    model = train.DPTrainModel(cfg, prm, davg, dstd, dtype=dtype, device=DEV)
    batch = {"list_neigh": torch.tensor(ln, device=DEV), "type_map": torch.tensor(st.types, device=DEV),
             "atom_type": cfg.atom_type, "ImageDR": torch.tensor(idr, device=DEV),
             "Etot": E_lab.to(DEV), "Force": F_lab.to(DEV)}
    tr = train.FusedTrainer(model)
    loss, _, _ = tr.loss_and_backward(batch)
    return model, loss


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-8), (torch.float32, 2e-3)])
def test_fused_training_gradients_match_oracle(dtype, tol):
    """Hand-written embedding double-backward (matpl_dp_dual_forward / _backward) + torch fitting
    part against second-order autograd through the FP64 oracle, every parameter."""
    case = make_case()
    loss_ref, g_ref = oracle_grads(*case)
    model, loss = _fused_grads(case, dtype)
    assert abs(loss - loss_ref) <= (1e-10 if dtype == torch.float64 else 1e-4) * abs(loss_ref)
    worst, where = 0.0, None
    for k, gr in g_ref.items():
        got = model.param(k).grad.detach().double().cpu()
        scale = gr.abs().max().item() + 1e-30
        err = (got - gr).abs().max().item() / scale
        if err > worst:
            worst, where = err, k
    print(f"[accuracy] fused training gradients {dtype}: worst relative error {worst:.2e} ({where})")
    assert worst < tol, (worst, where)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-11), (torch.float32, 2e-5)])
def test_fitting_kernel_matches_the_torch_fitting_part(dtype, tol):
    """matpl_dp_fit_dual (both streams and the reverse pass of the fitting nets in one kernel,
    the weight gradients as row sums) against the same mathematics as torch operations and
    autograd, every parameter; 600 atoms so that tiles and row chunks end part-way."""
    cfg, st, ln, idr, davg, dstd, prm, E_lab, F_lab = make_case(n=600, seed=13)
    batch = {"list_neigh": torch.tensor(ln, device=DEV), "type_map": torch.tensor(st.types, device=DEV),
             "atom_type": cfg.atom_type, "ImageDR": torch.tensor(idr, device=DEV),
             "Etot": E_lab.to(DEV), "Force": F_lab.to(DEV)}
    grads, losses = [], []
    for fk in (True, False):
        model = train.DPTrainModel(cfg, prm, davg, dstd, dtype=dtype, device=DEV)
        tr = train.FusedTrainer(model, fit_kernel=fk)
        assert tr.fit_kernel == fk
        loss, _, _ = tr.loss_and_backward(batch)
        losses.append(loss)
        grads.append({k: model.param(k).grad.detach().double().clone() for k in model.names})
    assert abs(losses[0] - losses[1]) <= (1e-12 if dtype == torch.float64 else 1e-6) * abs(losses[1])
    worst, where = 0.0, None
    for k, ref in grads[1].items():
        err = (grads[0][k] - ref).abs().max().item() / (ref.abs().max().item() + 1e-30)
        if err > worst:
            worst, where = err, k
    print(f"[accuracy] fitting kernel vs torch fitting part {dtype}: worst relative {worst:.2e} ({where})")
    assert worst < tol, (worst, where)


def test_fused_training_two_configs_and_fd():
    """Batch of two configurations of one composition, then a finite-difference check of the
    fused gradient of one embedding weight."""
    c1 = make_case(n=36, seed=7)
    c2 = make_case(n=36, seed=8)
    cfg, st, ln1, idr1, davg, dstd, prm, E1, F1 = c1
    ln2, idr2, E2, F2 = c2[2], c2[3], c2[7], c2[8]
    assert np.array_equal(c1[1].types, c2[1].types)
    model = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float64, device=DEV)
    batch = {"list_neigh": torch.tensor(np.concatenate([ln1, ln2]), device=DEV),
             "type_map": torch.tensor(st.types, device=DEV), "atom_type": cfg.atom_type,
             "ImageDR": torch.tensor(np.concatenate([idr1, idr2]), device=DEV),
             "Etot": torch.cat([E1, E2]).reshape(2, 1).to(DEV),
             "Force": torch.cat([F1, F2]).to(DEV)}
    ref_model = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float64, device=DEV)
    l_ref, _, _ = train.loss_fn(ref_model, batch)
    l_ref.backward()
    tr = train.FusedTrainer(model)
    loss, _, _ = tr.loss_and_backward(batch)
    assert abs(loss - l_ref.item()) <= 1e-10 * abs(l_ref.item())
    for k in model.names:
        a = model.param(k).grad
        b = ref_model.param(k).grad
        assert (a - b).abs().max().item() <= 1e-8 * (b.abs().max().item() + 1e-30), k
    name = "embedding_net.2.layers.2.weight"
    p = model.param(name)
    flat = p.detach().view(-1)
    q = 37
    h = 1e-6
    vals = []
    for sgn in (1, -1):
        with torch.no_grad():
            flat[q] += sgn * h
        vals.append(tr.loss_and_backward(batch)[0])
        with torch.no_grad():
            flat[q] -= sgn * h
    fd = (vals[0] - vals[1]) / (2 * h)
    model.zero_grad(set_to_none=True)
    tr.loss_and_backward(batch)
    got = model.param(name).grad.view(-1)[q].item()
    assert abs(fd - got) <= 1e-5 * max(1.0, abs(fd)), (fd, got)


def test_graphed_training_step_matches_eager():
    """The CUDA-graph-captured fused step gives the same parameters after a few SGD steps as
    the eager fused step (FP64)."""
    case = make_case(n=36, seed=7)
    cfg, st, ln, idr, davg, dstd, prm, E_lab, F_lab = case
    batch = {"list_neigh": torch.tensor(ln, device=DEV), "type_map": torch.tensor(st.types, device=DEV),
             "atom_type": cfg.atom_type, "ImageDR": torch.tensor(idr, device=DEV),
             "Etot": E_lab.to(DEV), "Force": F_lab.to(DEV)}
    m1 = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float64, device=DEV)
    m2 = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float64, device=DEV)
    o1 = torch.optim.SGD(m1.parameters(), lr=1e-5)
    o2 = torch.optim.SGD(m2.parameters(), lr=1e-5)
    t1 = train.FusedTrainer(m1)
    g2 = train.GraphedTrainer(train.FusedTrainer(m2), o2, warmup=2)
    for _ in range(2):                      # the graph's own warm-up steps
        t1.step([batch], o1)
    losses = []
    for _ in range(3):
        l1 = t1.step([batch], o1)
        l2 = g2.step(batch)
        losses.append((l1, float(l2)))
    for a, b in losses:
        assert abs(a - b) <= 1e-10 * abs(a)
    for k in m1.names:
        assert torch.allclose(m1.param(k), m2.param(k), rtol=1e-10, atol=1e-12), k


@pytest.mark.parametrize("m2,partial", [(16, False), (25, True), (4, False)])
def test_descriptor_product_kernel_matches_torch(m2, partial):
    """matpl_dp_desc_dual / _grad = torch's D = A^T A<, D_dot = A_dot^T A< + A^T A_dot< on the
    rows of a permutation (or a subset: the other atoms get zero gradient) and their autograd
    transpose (FP64, random A, A_dot, seeds; either seed absent)."""
    from matpl_gb300.train import _DescDual
    g = torch.Generator(device=DEV).manual_seed(m2)
    A = torch.randn(37, 4, 25, generator=g, device=DEV, dtype=torch.float64, requires_grad=True)
    Ad = torch.randn(37, 4, 25, generator=g, device=DEV, dtype=torch.float64, requires_grad=True)
    rows = torch.randperm(37, generator=g, device=DEV)
    if partial:
        rows = rows[:30]
    D, Dd = _DescDual.apply(A, Ad, m2, rows)
    Ar, Adr = A.index_select(0, rows), Ad.index_select(0, rows)
    Dr = Ar.transpose(-2, -1) @ Ar[..., :m2]
    Ddr = Adr.transpose(-2, -1) @ Ar[..., :m2] + Ar.transpose(-2, -1) @ Adr[..., :m2]
    torch.testing.assert_close(D, Dr, rtol=1e-13, atol=1e-13)
    torch.testing.assert_close(Dd, Ddr, rtol=1e-13, atol=1e-13)
    gD = torch.randn(D.shape, generator=g, device=DEV, dtype=torch.float64)
    gDd = torch.randn(D.shape, generator=g, device=DEV, dtype=torch.float64)
    for seeds in ((gD, gDd), (gD, None), (None, gDd)):
        outs = [o for o, s in zip((D, Dd), seeds) if s is not None]
        refs = [o for o, s in zip((Dr, Ddr), seeds) if s is not None]
        gs = [s for s in seeds if s is not None]
        k = torch.autograd.grad(outs, [A, Ad], gs, retain_graph=True, allow_unused=True)
        r = torch.autograd.grad(refs, [A, Ad], gs, retain_graph=True, allow_unused=True)
        for a, b in zip(k, r):
            a = torch.zeros_like(A) if a is None else a
            b = torch.zeros_like(A) if b is None else b
            torch.testing.assert_close(a, b, rtol=1e-12, atol=1e-12)


def _empty_slot_term_torch(model, ln, tm, present, davg4, dstd4):
    """The empty-slot term of A restated with torch operations on the model's Parameters: every
    empty slot of type block t_j holds the normalised zero row R_pad(t_i) = -davg / dstd, so it
    adds R_pad^T G_{t_i t_j}(R_pad[0]) once per empty slot, scaled by 1 / (m npresent)."""
    cfg = model.cfg
    T, m = cfg.ntypes, cfg.maxNeighborNum
    B, N, S = ln.shape
    occ = (ln > 0).reshape(B, N, T, m).sum(-1)
    out = torch.zeros(B, N, 4, 25, dtype=model.dtype, device=ln.device)
    for ti in present:
        rp = (0.0 - davg4[ti]) / dstd4[ti]
        for tj in present:
            G = model._emb(ti * T + tj, rp[0].reshape(1, 1))
            row = rp.reshape(4, 1) * G.reshape(1, 25)
            w = (tm == ti).reshape(1, N, 1, 1).to(model.dtype) * \
                (m - occ[:, :, tj]).to(model.dtype).reshape(B, N, 1, 1)
            out = out + w * row
    return out / (m * len(present))


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 2e-5)])
@pytest.mark.parametrize("present", [[0, 1], [1, 0], [1]])
def test_empty_slot_kernels_match_torch(dtype, tol, present):
    """matpl_dp_pad_forward / _backward against the torch restatement: A = A_occ + the term
    (atoms of a type absent from present[] copy A_occ), and the embedding-parameter gradient of
    <A, seed> through it, for two configurations of 300 atoms."""
    cfg, st, ln, idr, davg, dstd, prm, _, _ = make_case(n=300, seed=17)
    model = train.DPTrainModel(cfg, prm, davg, dstd, dtype=dtype, device=DEV)
    tr = train.FusedTrainer(model)
    tr._present = list(present)
    ln_d = torch.tensor(ln, device=DEV).to(torch.int32)
    ln_d = torch.cat([ln_d, ln_d.flip(-1)], 0).contiguous()       # second config: other counts
    tm = torch.tensor(st.types, device=DEV).to(torch.int32)
    B, N, S = ln_d.shape
    g = torch.Generator(device=DEV).manual_seed(3)
    A_occ = torch.randn(B * N, 100, generator=g, device=DEV, dtype=dtype)
    seed = torch.randn(B * N, 100, generator=g, device=DEV, dtype=dtype)
    A = train._EmptySlots.apply(A_occ, train._emb_flat(model), tr, ln_d, tm)
    ref = _empty_slot_term_torch(model, ln_d, tm.long(), present, tr.davg4, tr.dstd4)
    torch.testing.assert_close(A - A_occ, ref.reshape(B * N, 100), rtol=tol, atol=tol)
    absent = ~torch.isin(tm.long(), torch.tensor(present, device=DEV))
    if absent.any():
        rows = absent.repeat(B)
        assert torch.equal(A[rows], A_occ[rows])
    params = [model.param(k) for k in model.names]
    gk = torch.autograd.grad((A * seed).sum(), params, allow_unused=True)
    gr = torch.autograd.grad((ref.reshape(B * N, 100) * seed).sum(), params, allow_unused=True)
    worst = 0.0
    for k, a, b in zip(model.names, gk, gr):
        if not k.startswith("embedding_net."):
            assert a is None or not a.any(), k
            continue
        a = torch.zeros_like(model.param(k)) if a is None else a
        b = torch.zeros_like(model.param(k)) if b is None else b
        worst = max(worst, ((a - b).abs().max() / (b.abs().max() + 1e-30)).item()
                    if b.abs().max() > 0 else a.abs().max().item())
    print(f"[accuracy] empty-slot kernels {dtype} present={present}: worst relative {worst:.2e}")
    assert worst < tol, worst
