"""Type-embedding DP on the GPU against MatPL's own TypeDP (golden from its CPU branch):
E, Ei, forces, virial and the training gradient of an energy + force loss."""
import numpy as np
import pytest
import torch

from matpl_gb300.typedp import TypeDP, init_type_params

pytestmark = pytest.mark.gpu
DEV = "cuda"


def test_typedp_matches_reference(golden_case):
    from tests.conftest import load_golden
    g = load_golden("typedp_hfo48")
    c = golden_case("hfo48_f64")
    cfg = c.cfg
    vec = {z: list(v) for z, v in zip(cfg.atom_type, g["type_vector"])}
    params = init_type_params(cfg, g["type_vector"].shape[1], int(g["seed_w"]))
    model = TypeDP(cfg, params, c.davg, c.dstd, vec, device=DEV)
    Etot, Ei, F, V = model(torch.tensor(c.list_neigh, device=DEV),
                           torch.tensor(c.types, device=DEV), cfg.atom_type,
                           torch.tensor(c.image_dr, device=DEV), 0)
    np.testing.assert_allclose(Etot.detach().cpu().numpy().ravel(), g["Etot"].ravel(), rtol=1e-11)
    np.testing.assert_allclose(Ei.detach().cpu().numpy(), g["Ei"].reshape(Ei.shape), rtol=0,
                               atol=1e-11)
    fs = np.abs(g["Force"]).max()
    np.testing.assert_allclose(F.detach().cpu().numpy(), g["Force"], rtol=0, atol=1e-10 * fs)
    vs = np.abs(g["Virial"]).max()
    np.testing.assert_allclose(V.detach().cpu().numpy(), g["Virial"], rtol=0, atol=1e-9 * vs)
    rng = np.random.default_rng(int(g["seed_g"]))
    gE = rng.standard_normal(1)
    gF = rng.standard_normal(tuple(F.shape))
    L = (torch.tensor(gE, device=DEV) * Etot.reshape(-1)).sum() + \
        (torch.tensor(gF, device=DEV) * F).sum()
    L.backward()
    for name in model.names:
        ref = g["grad:" + name]
        got = model.param(name).grad.detach().cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * max(1.0, np.abs(ref).max()))


def test_typedp_fused_matches_reference(golden_case):
    """TypeDP in the fused kernels (v(t_j) folded into the first layer's bias of per-pair
    nets): FP64 = the reference's TypeDP (golden) to 1e-10; FP32 and the BF16x3 tcgen05 form
    within 1e-5 eV/atom (energy) and 1e-5 of the force scale (the BF16x3 form: or 1e-6 eV/A,
    whichever is larger)."""
    from matpl_gb300.typedp import fused_model
    from tests.conftest import load_golden
    g = load_golden("typedp_hfo48")
    c = golden_case("hfo48_f64")
    cfg = c.cfg
    vec = {z: list(v) for z, v in zip(cfg.atom_type, g["type_vector"])}
    params = init_type_params(cfg, g["type_vector"].shape[1], int(g["seed_w"]))
    ln = torch.tensor(c.list_neigh, device=DEV)
    tm = torch.tensor(c.types, device=DEV)
    idr = torch.tensor(c.image_dr, device=DEV)
    fs, vs = np.abs(g["Force"]).max(), np.abs(g["Virial"]).max()
    for prec, tol in (("float64", 1e-10), ("float32", 1e-5), ("mixed", 1e-5)):
        m = fused_model(cfg, params, c.davg, c.dstd, vec, precision=prec, device=DEV)
        Etot, Ei, F, _, V = m(ln, tm, cfg.atom_type, idr if prec == "float64" else idr.float(), 0)
        E = Etot.detach().double().cpu().numpy().ravel()
        Fn = F.detach().double().cpu().numpy().reshape(g["Force"].shape)
        print(f"[accuracy] typedp fused {prec}: E/atom {np.abs(E - g['Etot'].ravel()).max() / 48:.2e}"
              f" max|dF| {np.abs(Fn - g['Force']).max():.2e}")
        if prec == "float64":
            np.testing.assert_allclose(E, g["Etot"].ravel(), rtol=1e-11)
        else:
            assert np.abs(E - g["Etot"].ravel()).max() <= 1e-5 * 48
        # the BF16x3 form keeps per-pair terms to 2^-16 relative (two-part split), an absolute
        # floor of ~1e-6 eV/A once they cancel; this weakly forced cell has max|F| ~ 0.04 eV/A
        f_atol = max(tol * fs, 1e-6) if prec == "mixed" else tol * fs
        np.testing.assert_allclose(F.detach().double().cpu().numpy().reshape(g["Force"].shape),
                                   g["Force"], rtol=0, atol=f_atol)
        np.testing.assert_allclose(V.detach().double().cpu().numpy().reshape(g["Virial"].shape),
                                   g["Virial"], rtol=0, atol=10 * tol * vs)
