"""Data path on the GPU: matpl_env_stats against the oracle sums, and the davg / dstd of
set_davg_dstd against MatPL's own loader (golden fixture)."""
import random

import numpy as np
import pytest
import torch

from matpl_gb300 import data as D, structures
from oracle import neigh
from tests.test_data_path import cfg_of, cpu_stats, golden_images, load

pytestmark = pytest.mark.gpu


def test_env_stats_match_oracle_sums():
    g = load()
    cfg = cfg_of(g)
    ims = golden_images()
    ims = ims + [ims[0], ims[1]]          # repeated shapes run as one batch
    gpu = D.image_stats(cfg, ims)
    cpu = cpu_stats(cfg, ims)
    for a, b in zip(gpu, cpu):
        assert a["types"] == b["types"] and a["counts"] == b["counts"]
        np.testing.assert_allclose(a["sums"], b["sums"], rtol=1e-12, atol=1e-14)


def test_set_davg_dstd_on_gpu_matches_loader():
    g = load()
    cfg = cfg_of(g)
    davg, dstd = D.set_davg_dstd(cfg, golden_images(), rng=random.Random(int(g["seed_shuffle"])))
    np.testing.assert_allclose(davg, g["davg"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(dstd, g["dstd"], rtol=1e-12, atol=1e-15)


def test_env_stats_large_batch():
    """256 Cu images of 108 atoms in one launch: sums = the oracle's for a few of them."""
    from matpl_gb300 import params as P
    cfg = P.DPConfig(atom_type=[29], maxNeighborNum=100)
    ims = [structures.fcc(3.615, (3, 3, 3), 0.08, seed=s) for s in range(256)]
    gpu = D.image_stats(cfg, ims)
    for k in (0, 100, 255):
        ref = cpu_stats(cfg, [ims[k]])[0]
        np.testing.assert_allclose(gpu[k]["sums"], ref["sums"], rtol=1e-12, atol=1e-14)
