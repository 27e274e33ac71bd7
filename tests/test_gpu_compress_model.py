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


@pytest.mark.parametrize("order", [5, 3])
def test_fused_compressed_matches_reference(golden_case, order):
    """The table in the fused kernels (matpl_dp_eval with ctable): FP64 = the reference's
    compressed model (golden) and the operator path (CompressedDP) to 1e-10; FP32 within 1e-5 of
    the force scale, the mixed form (fitting nets on the tensor cores) within 1e-5 eV/A and
    1e-5 eV/atom."""
    g = load("compress_hfo48")
    c = golden_case("hfo48_f64")
    cfg = c.cfg
    comp = C.build_table(cfg, c.params, c.davg.numpy(), c.dstd.numpy(), float(g["sij_max_raw"]),
                         float(g["dx"]), order)
    ln = torch.tensor(c.list_neigh, device=DEV)
    idr = torch.tensor(c.image_dr, device=DEV)
    tm = torch.tensor(c.types, device=DEV)
    ref = C.CompressedDP(cfg, c.params, c.davg, c.dstd, comp, device=DEV)
    rE, _, rF, rV = ref(ln, tm, cfg.atom_type, idr, 0)
    rE, rF, rV = (x.detach().cpu().numpy() for x in (rE, rF, rV))
    fs = np.abs(g[f"o{order}_Force"]).max()
    vs = np.abs(g[f"o{order}_Virial"]).max()
    model = C.fused_model(cfg, c.params, c.davg, c.dstd, comp, "float64", DEV)
    Etot, Ei, F, _, V = model(ln, tm, cfg.atom_type, idr, 0)
    Etot, F, V = (x.detach().cpu().numpy() for x in (Etot, F, V))
    np.testing.assert_allclose(Etot.ravel(), g[f"o{order}_Etot"].ravel(), rtol=1e-11)
    np.testing.assert_allclose(F.reshape(rF.shape), g[f"o{order}_Force"], rtol=0, atol=1e-10 * fs)
    np.testing.assert_allclose(V.reshape(rV.shape), g[f"o{order}_Virial"], rtol=0, atol=1e-9 * vs)
    np.testing.assert_allclose(Etot.ravel(), rE.ravel(), rtol=1e-12)
    np.testing.assert_allclose(F.reshape(rF.shape), rF, rtol=0, atol=1e-10 * fs)
    np.testing.assert_allclose(Ei.detach().sum().item(), rE.sum(), rtol=1e-12)
    m32 = C.fused_model(cfg, c.params, c.davg, c.dstd, comp, "float32", DEV)
    E32, _, F32, _, V32 = m32(ln, tm, cfg.atom_type, idr.float(), 0)
    np.testing.assert_allclose(E32.detach().cpu().numpy().ravel(), g[f"o{order}_Etot"].ravel(),
                               rtol=1e-5)
    np.testing.assert_allclose(F32.detach().cpu().numpy().reshape(rF.shape), g[f"o{order}_Force"],
                               rtol=0, atol=1e-5 * fs)
    # the mixed forms: table in the SIMT embedding kernels, fitting nets on the tensor cores
    mx = C.fused_model(cfg, c.params, c.davg, c.dstd, comp, "mixed", DEV)
    Em, _, Fm, _, _ = mx(ln, tm, cfg.atom_type, idr.float(), 0)
    natoms = c.list_neigh.shape[1]
    assert abs(Em.item() - float(g[f"o{order}_Etot"].ravel()[0])) <= 1e-5 * natoms
    np.testing.assert_allclose(Fm.detach().cpu().numpy().reshape(rF.shape), g[f"o{order}_Force"],
                               rtol=0, atol=1e-5)         # eV/A (this cell's forces are < 0.1)
    assert int(model.err.item()) == 0 and int(m32.err.item()) == 0 and int(mx.err.item()) == 0
