"""Compressed DP on the GPU against MatPL's compressed model (golden: the reference DP with the
reference's own table, CPU compress branch): E, Ei, forces, virial for orders 5 and 3, with the
table from this library's builder."""
import numpy as np
import pytest
import torch

from matpl_gb300 import compress as C, ops, params as P

pytestmark = pytest.mark.gpu
DEV = "cuda"


def load(name):
    from tests.conftest import load_golden
    return load_golden(name)


@pytest.mark.parametrize("order", [5, 3])
def test_compressed_model_matches_reference(golden_case, order):
    g = load("compress_hfo48")
    c = golden_case("hfo48_f64")
    cfg = c.cfg
    comp = C.build_table(cfg, c.params, c.davg.numpy(), c.dstd.numpy(), float(g["sij_max_raw"]),
                         float(g["dx"]), order)
    model = C.CompressedDP(cfg, c.params, c.davg, c.dstd, comp, device=DEV)
    ln = torch.tensor(c.list_neigh, device=DEV)
    idr = torch.tensor(c.image_dr, device=DEV)
    tm = torch.tensor(c.types, device=DEV)
    Etot, Ei, F, V = model(ln, tm, cfg.atom_type, idr, 0)
    np.testing.assert_allclose(Etot.detach().cpu().numpy().ravel(), g[f"o{order}_Etot"].ravel(),
                               rtol=1e-11)
    np.testing.assert_allclose(Ei.detach().cpu().numpy(), g[f"o{order}_Ei"].reshape(Ei.shape),
                               rtol=0, atol=1e-11)
    fs = np.abs(g[f"o{order}_Force"]).max()
    np.testing.assert_allclose(F.detach().cpu().numpy(), g[f"o{order}_Force"], rtol=0,
                               atol=1e-10 * fs)
    vs = np.abs(g[f"o{order}_Virial"]).max()
    np.testing.assert_allclose(V.detach().cpu().numpy(), g[f"o{order}_Virial"], rtol=0,
                               atol=1e-9 * vs)


def test_compressed_close_to_exact_with_correct_widths(golden_case):
    """With every pair's own interval widths the order-5 table reproduces the exact nets."""
    g = load("compress_hfo48")
    c = golden_case("hfo48_f64")
    comp = C.build_table(c.cfg, c.params, c.davg.numpy(), c.dstd.numpy(),
                         float(g["sij_max_raw"]), float(g["dx"]), 5, reference_dx_growth=False)
    model = C.CompressedDP(c.cfg, c.params, c.davg, c.dstd, comp, device=DEV)
    Etot, _, F, _ = model(torch.tensor(c.list_neigh, device=DEV), torch.tensor(c.types, device=DEV),
                          c.cfg.atom_type, torch.tensor(c.image_dr, device=DEV), 0)
    np.testing.assert_allclose(Etot.item(), c.g["Etot"].item(), rtol=1e-7)
    np.testing.assert_allclose(F.detach().cpu().numpy(), c.g["Force"], rtol=0,
                               atol=1e-5 * np.abs(c.g["Force"]).max())
