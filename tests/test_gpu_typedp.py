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
