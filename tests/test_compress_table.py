"""The compression table builder against MatPL's own (golden from ckpt_compress.py run on the
reference DP): grid, shape and coefficients for orders 5 and 3."""
import numpy as np
import pytest

from matpl_gb300 import compress as C, params as P


def load(name):
    from tests.conftest import load_golden
    return load_golden(name)


@pytest.mark.parametrize("order", [5, 3])
def test_table_matches_reference(order):
    g = load("compress_hfo48")
    base = load("hfo48_f64")
    cfg = P.DPConfig(atom_type=[int(a) for a in base["atom_type"]], maxNeighborNum=int(base["m"]),
                     Rmax=float(base["Rmax"]), Rmin=float(base["Rmin"]))
    comp = C.build_table(cfg, P.init_params(cfg, int(base["seed_w"])), base["davg"], base["dstd"],
                         float(g["sij_max_raw"]), float(g["dx"]), order)
    assert np.array_equal(np.array(comp["table"].shape), g[f"o{order}_shape"])
    grid = np.array([comp["sij_min"], comp["sij_max"], comp["sij_out_max"], comp["sij_len"],
                     comp["sij_out_len"]])
    np.testing.assert_allclose(grid, g[f"o{order}_grid"], rtol=1e-15)
    sample = comp["table"][:, g[f"o{order}_rows"]]
    ref = g[f"o{order}_sample"]
    np.testing.assert_allclose(sample, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
