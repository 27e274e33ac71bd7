"""Data path on the CPU: davg / dstd arithmetic and image selection, energy shift and batch
grouping against golden values from MatPL's own loader functions (calc_stat,
UniDataset.set_davg_dstd / set_energy_shift, run in this container with the neighbor lists of
the oracle restatement of NeighConst)."""
import random

import numpy as np
import pytest
import torch

from matpl_gb300 import data as D, params as P, structures
from oracle import neigh


def load():
    from tests.conftest import load_golden
    return load_golden("data_stats")


def golden_images():
    import importlib.util
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                        "make_data_golden.py")
    spec = importlib.util.spec_from_file_location("make_data_golden", here)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.images()


def cfg_of(g):
    return P.DPConfig(atom_type=[int(a) for a in g["atom_type"]], maxNeighborNum=int(g["m"]),
                      Rmax=float(g["Rc"]), Rmin=float(g["Rmin"]))


def cpu_stats(cfg, images):
    """image_stats with the oracle's neighbor lists and sums (no GPU)."""
    out = []
    for st in images:
        tm = D.model_types(st, cfg.atom_type)
        ln, idr = neigh.find_neighbore(tm, st.frac, st.lattice, cfg.ntypes, cfg.maxNeighborNum,
                                       cfg.Rmax, [cfg.Rmax] * cfg.ntypes)
        sums = neigh.env_sums(cfg, ln, idr, tm)[0]
        _, first, counts = np.unique(tm, return_index=True, return_counts=True)
        order = np.argsort(first)
        out.append({"types": np.unique(tm)[order].tolist(), "counts": counts[order].tolist(),
                    "sums": sums})
    return out


def test_stat_units_match_calc_stat():
    g = load()
    cfg = cfg_of(g)
    ims = golden_images()
    for k, rec in enumerate(cpu_stats(cfg, ims)):
        davg, dstd = D.stat_units(cfg, rec)
        np.testing.assert_allclose(davg, g[f"img{k}_davg"], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(dstd, g[f"img{k}_dstd"], rtol=1e-12, atol=1e-15)


def test_set_davg_dstd_picks_like_the_loader():
    g = load()
    cfg = cfg_of(g)
    davg, dstd = D.set_davg_dstd(cfg, golden_images(), rng=random.Random(int(g["seed_shuffle"])),
                                 stats_fn=cpu_stats)
    assert davg.shape == (cfg.ntypes, cfg.ntypes * cfg.maxNeighborNum * 4)
    np.testing.assert_allclose(davg, g["davg"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(dstd, g["dstd"], rtol=1e-12, atol=1e-15)


def test_energy_shift_matches_loader():
    g = load()
    shift = D.set_energy_shift(golden_images(), g["energies"], [int(a) for a in g["atom_type"]],
                               rng=random.Random(int(g["seed_shuffle"])))
    np.testing.assert_allclose(shift, g["energy_shift"], rtol=1e-12)


def test_classify_and_uniform_batches():
    tmaps = torch.tensor([[0, 0, 1, -1], [0, 1, 0, -1], [1, 1, 1, 1], [0, 0, 1, -1]])
    assert D.classify_batches(tmaps, 2) == [[0, 1, 3], [2]]
    ims = golden_images()
    groups = D.uniform_batches(ims + ims[:3], [3, 14], max_batch=2)
    seen = sorted(k for grp in groups for k in grp)
    assert seen == list(range(len(ims) + 3))
    for grp in groups:
        assert len(grp) <= 2
        allims = ims + ims[:3]
        keys = {(allims[k].natoms, tuple(D.model_types(allims[k], [3, 14]).tolist())) for k in grp}
        assert len(keys) == 1
