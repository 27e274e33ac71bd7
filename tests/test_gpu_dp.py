"""Fused DP se_e2_a E/F/V on the GPU against the reference's own outputs (golden fixtures
from MatPL's DP implementation and its shipped TorchScript model) and the oracle."""
import numpy as np
import pytest
import torch

from matpl_gb300 import dp, ops, params as P, structures
from oracle import dp_oracle, neigh

pytestmark = pytest.mark.gpu
DEV = "cuda"
GOLDEN = ["cu108_f64", "cu108_f32", "cu108x2_f64", "lisi600_f64", "hfo48_f64", "hfo2_jit"]


def run_model(c, precision):
    m = dp.DP(c.cfg, c.params, c.davg, c.dstd, precision=precision, device=DEV)
    dt = m.dtype
    return m(torch.tensor(c.list_neigh, device=DEV), torch.tensor(c.types, device=DEV),
             torch.tensor(c.cfg.atom_type), torch.tensor(c.image_dr, dtype=dt, device=DEV), 0)


@pytest.mark.parametrize("name", GOLDEN)
def test_dp_matches_reference_golden(golden_case, name):
    """E, Ei (type-grouped), F within 1e-10 relative of the reference in FP64."""
    c = golden_case(name)
    g = c.g
    prec = "float64" if c.dtype == torch.float64 else "float32"
    Etot, Ei, F, _, V = run_model(c, prec)
    tol = 1e-10 if prec == "float64" else 2e-5
    np.testing.assert_allclose(Etot.cpu().numpy().ravel(), g["Etot"].ravel(), rtol=tol)
    np.testing.assert_allclose(Ei.cpu().numpy(), g["Ei"].reshape(Ei.shape), rtol=0,
                               atol=tol * np.abs(g["Ei"]).max())
    fs = np.abs(g["Force"]).max()
    np.testing.assert_allclose(F.cpu().numpy(), g["Force"], rtol=0, atol=tol * fs * 10)
    # reference CPU virial is the mirrored upper triangle; ours is the full f_a R_c matrix
    vs = np.abs(g["Virial"]).max()
    np.testing.assert_allclose(V.cpu().numpy(), g["Virial"], rtol=0, atol=tol * vs * 10)


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_dp_matches_oracle_full_virial(golden_case, precision):
    c = golden_case("hfo2_jit")
    dt = torch.float64 if precision == "float64" else torch.float32
    ref = dp_oracle.dp_eval(c.cfg, {k: v.to(dt) for k, v in c.params.items()}, c.davg, c.dstd,
                            torch.tensor(c.list_neigh), torch.tensor(c.types),
                            torch.tensor(c.cfg.atom_type), torch.tensor(c.image_dr, dtype=dt), 0,
                            virial_convention="gpu")
    Etot, Ei, F, _, V = run_model(c, precision)
    tol = 1e-10 if precision == "float64" else 3e-5
    np.testing.assert_allclose(V.cpu().numpy(), ref["Virial"].detach().numpy(), rtol=0,
                               atol=tol * ref["Virial"].abs().max().item() * 10)


def test_dp_ghost_atoms_and_absent_types(golden_case):
    """nghost > 0 (LAMMPS) routes neighbor forces to ghost rows; an image lacking one model
    type evaluates only the present type (dp_dp.py:145-165, 354-372)."""
    c = golden_case("hfo2_jit")
    ln = torch.tensor(c.list_neigh)
    N = ln.shape[1]
    nghost = 5
    ln_g = torch.where((ln > 0) & (ln % 3 == 0), N + 1 + (ln % nghost), ln)
    ref = dp_oracle.dp_eval(c.cfg, c.params, c.davg, c.dstd, ln_g, torch.tensor(c.types),
                            torch.tensor(c.cfg.atom_type), torch.tensor(c.image_dr), nghost)
    m = dp.DP(c.cfg, c.params, c.davg, c.dstd, device=DEV)
    Etot, Ei, F, _, V = m(ln_g.to(DEV), torch.tensor(c.types, device=DEV),
                          torch.tensor(c.cfg.atom_type), torch.tensor(c.image_dr, device=DEV), nghost)
    assert F.shape == (1, N + nghost, 3)
    np.testing.assert_allclose(F.cpu().numpy(), ref["Force"].detach().numpy(), rtol=0, atol=1e-10)
    # only Hf (model type 1) present in the image type list
    at = torch.tensor([c.cfg.atom_type[1]])
    ref2 = dp_oracle.dp_eval(c.cfg, c.params, c.davg, c.dstd, torch.tensor(c.list_neigh),
                             torch.tensor(c.types), at, torch.tensor(c.image_dr), 0)
    E2, Ei2, F2, _, _ = m(torch.tensor(c.list_neigh, device=DEV), torch.tensor(c.types, device=DEV),
                          at, torch.tensor(c.image_dr, device=DEV), 0)
    np.testing.assert_allclose(E2.cpu().numpy().ravel(), ref2["Etot"].detach().numpy().ravel(),
                               rtol=1e-10)
    np.testing.assert_allclose(F2.cpu().numpy(), ref2["Force"].detach().numpy(), rtol=0, atol=1e-10)


def test_forces_are_minus_energy_gradient():
    """Central finite differences of E (FP64, GPU path end to end incl. neighbor rebuild)."""
    st = structures.random_packed(60, 0.07, [72, 8], [1 / 3, 2 / 3], seed=8, strain=0.03)
    cfg = P.DPConfig(atom_type=[72, 8], maxNeighborNum=120)
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, 120, 6.0, [6.0, 6.0])
    davg, dstd = P.calc_stat(cfg, ln, idr, st.types)
    m = dp.DP(cfg, P.init_params(cfg, 5), davg, dstd, device=DEV)
    tm = torch.tensor(st.types, device=DEV)
    at = torch.tensor(cfg.atom_type)

    def energy_force(cart):
        frac = np.mod(cart @ np.linalg.inv(st.lattice), 1.0)
        l, r = ops.find_neighbore(torch.tensor(st.types), torch.tensor(frac, device=DEV),
                                  torch.tensor(st.lattice), 2, 120, 6.0, 6.0)
        E, _, F, _, _ = m(l, tm, at, r, 0)
        return E.item(), F[0].cpu().numpy()

    cart = st.cart
    _, F0 = energy_force(cart)
    h = 1e-5
    rng = np.random.default_rng(0)
    for a in rng.choice(len(cart), 6, replace=False):
        for k in range(3):
            cp, cm = cart.copy(), cart.copy()
            cp[a, k] += h
            cm[a, k] -= h
            fd = -(energy_force(cp)[0] - energy_force(cm)[0]) / (2 * h)
            assert abs(fd - F0[a, k]) < 1e-6 * max(1.0, abs(F0[a, k])), (a, k, fd, F0[a, k])


def test_virial_is_strain_derivative():
    """V = -dE/d(eps) under homogeneous strain (MatPL convention: virial = sum r (x) f)."""
    st = structures.random_packed(60, 0.07, [72, 8], [1 / 3, 2 / 3], seed=9)
    cfg = P.DPConfig(atom_type=[72, 8], maxNeighborNum=120)
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, 120, 6.0, [6.0, 6.0])
    davg, dstd = P.calc_stat(cfg, ln, idr, st.types)
    m = dp.DP(cfg, P.init_params(cfg, 6), davg, dstd, device=DEV)
    tm = torch.tensor(st.types, device=DEV)
    at = torch.tensor(cfg.atom_type)

    def ev(lat):
        l, r = ops.find_neighbore(torch.tensor(st.types), torch.tensor(st.frac, device=DEV),
                                  torch.tensor(lat), 2, 120, 6.0, 6.0)
        E, _, _, _, V = m(l, tm, at, r, 0)
        return E.item(), V[0].cpu().numpy().reshape(3, 3)

    _, V0 = ev(st.lattice)
    h = 1e-6
    for a in range(3):
        for b in range(3):
            eps = np.zeros((3, 3))
            eps[a, b] = h
            Ep = ev(st.lattice @ (np.eye(3) + eps))[0]
            Em = ev(st.lattice @ (np.eye(3) - eps))[0]
            dEde = (Ep - Em) / (2 * h)
            # E(r (I+eps)): dE/deps_ab = sum_k dE/dr_ka r_kb -> -sum r_b f_a
            assert abs(dEde + V0[a, b]) < 1e-5 * max(1.0, np.abs(V0).max()), (a, b, dEde, V0[a, b])


def test_full_size_32k_invariants():
    """Config of the headline metric: 32,000 Li/Si atoms, m = 150 per type.  Net force ~ 0,
    virial symmetric, FP32 vs FP64 force RMSE small."""
    st = structures.random_packed(32000, 0.05, [3, 14], [0.5, 0.5], seed=2024)
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150)
    ln, idr = ops.find_neighbore(torch.tensor(st.types), torch.tensor(st.frac, device=DEV),
                                 torch.tensor(st.lattice), 2, 150, 6.0, 6.0)
    sub = slice(0, 2000)
    davg, dstd = P.calc_stat(cfg, ln[:, sub].cpu().numpy(), idr[:, sub].cpu().numpy(), st.types[sub])
    prm = P.init_params(cfg, 11)
    tm = torch.tensor(st.types, device=DEV)
    at = torch.tensor(cfg.atom_type)
    m64 = dp.DP(cfg, prm, davg, dstd, precision="float64", device=DEV)
    m32 = dp.DP(cfg, prm, davg, dstd, precision="float32", device=DEV)
    E64, _, F64, _, V64 = m64(ln, tm, at, idr, 0)
    E32, _, F32, _, V32 = m32(ln, tm, at, idr.float(), 0)
    F64 = F64[0].double()
    assert F64.sum(0).abs().max().item() < 1e-9 * F64.abs().max().item() * 32000
    Vm = V64[0].reshape(3, 3)
    assert (Vm - Vm.t()).abs().max().item() < 1e-9 * Vm.abs().max().item()
    rmse = (F32[0].double() - F64).pow(2).mean().sqrt().item()
    assert rmse < 1e-4, rmse
    assert abs(E32.item() - E64.item()) < 1e-5 * abs(E64.item()) + 1e-3


MIXED = ["mixed", "mixed_fast", "mixed_tanhf"]


@pytest.mark.parametrize("precision", MIXED)
@pytest.mark.parametrize("name", ["cu108_f64", "lisi600_f64", "hfo2_jit"])
def test_mixed_forms_within_tolerance_of_reference(golden_case, precision, name):
    """tcgen05 forms: force RMSE <= 1e-4 eV/A against the reference FP64 forces; energy and
    virial close (error stated per form)."""
    c = golden_case(name)
    g = c.g
    Etot, Ei, F, _, V = run_model(c, precision)
    rmse = np.sqrt(np.mean((F.cpu().double().numpy() - g["Force"]) ** 2))
    # BF16x3 forms stay within 1e-4 eV/A; the single-BF16 embedding form carries ~1 % relative
    # force error (2.5e-3 eV/A on the reference's HfO2 weights), reported but not held to the bar
    fmax = np.abs(g["Force"]).max()
    n = c.types.shape[0]
    e_err = abs(Etot.item() - g["Etot"].ravel()[0]) / n
    vs = max(1.0, np.abs(g["Virial"]).max())
    v_err = np.abs(V.cpu().double().numpy() - g["Virial"]).max() / vs
    print(f"[accuracy] {precision} {name}: force RMSE {rmse:.3e} eV/A (max|F| {fmax:.3f}), "
          f"energy {e_err:.3e} eV/atom, virial {v_err:.3e} relative")
    if precision == "mixed_tanhf":    # BF16x3 + tanhf: FP32-level
        assert rmse <= 3e-5 and e_err < 2e-6 and v_err < 5e-5, (rmse, e_err, v_err)
    elif precision == "mixed":        # BF16x3 + hardware tanh: within the 1e-4 eV/A bar
        assert rmse <= 1e-4 and e_err < 2e-4 and v_err < 2e-3, (rmse, e_err, v_err)
    else:                             # single BF16: sanity only (about 1 % relative error)
        assert rmse <= 0.02 * fmax and e_err < 2e-2 and v_err < 5e-2, (rmse, e_err, v_err)


@pytest.mark.parametrize("precision", MIXED)
def test_mixed_forms_full_size(precision):
    """32,000-atom Li/Si box: force RMSE against the FP64 GPU path (itself pinned to the
    reference) stays within 1e-4 eV/A, net force ~ 0, no kernel error."""
    st = structures.random_packed(32000, 0.05, [3, 14], [0.5, 0.5], seed=2024)
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150)
    ln, idr = ops.find_neighbore(torch.tensor(st.types), torch.tensor(st.frac, device=DEV),
                                 torch.tensor(st.lattice), 2, 150, 6.0, 6.0)
    sub = slice(0, 2000)
    davg, dstd = P.calc_stat(cfg, ln[:, sub].cpu().numpy(), idr[:, sub].cpu().numpy(), st.types[sub])
    prm = P.init_params(cfg, 11)
    tm = torch.tensor(st.types, device=DEV)
    at = torch.tensor(cfg.atom_type)
    E64, _, F64, _, V64 = dp.DP(cfg, prm, davg, dstd, precision="float64", device=DEV)(ln, tm, at, idr, 0)
    m = dp.DP(cfg, prm, davg, dstd, precision=precision, device=DEV)
    E, _, F, _, V = m(ln, tm, at, idr.float(), 0)
    rmse = (F[0].double() - F64[0]).pow(2).mean().sqrt().item()
    e_err = abs(E.item() - E64.item()) / 32000
    print(f"[accuracy] {precision} 32k Li/Si: force RMSE {rmse:.3e} eV/A, energy {e_err:.3e} eV/atom")
    if precision != "mixed_fast":
        assert rmse <= 1e-4, rmse
        assert e_err < 2e-4, e_err
    else:
        assert rmse <= 0.02 * F64[0].abs().max().item(), rmse
    assert F[0].double().sum(0).abs().max().item() < 1e-2


def test_autotuner_sets_tile_shape_without_changing_results(golden_case):
    """The mixed kernels' tile shape (centre atoms per CTA group, CTAs per SM) is timed by the
    autotuner, which keeps the fastest; forces are the same for every candidate."""
    from matpl_gb300 import autotune, dp
    c = golden_case("lisi600_f64")
    model = dp.DP(c.cfg, c.params, c.davg, c.dstd, precision="mixed", device="cuda")
    ln = torch.tensor(c.list_neigh, device="cuda")
    idr = torch.tensor(c.image_dr, device="cuda", dtype=torch.float32)
    tm = torch.tensor(c.types, device="cuda", dtype=torch.int32)
    present = model.present_types(c.cfg.atom_type)
    try:
        res = autotune.tune_dp_mixed(model, ln, tm, present, idr, groups=(2, 7, 16), ctas=(1, 3),
                                     reps=2)
        assert len(res["table"]) == 6
        assert autotune.get_tuning() == (res["group_atoms"], res["ctas_per_sm"])
    finally:
        autotune.set_tuning(0, 0)
    assert autotune.get_tuning() == (0, 0)
