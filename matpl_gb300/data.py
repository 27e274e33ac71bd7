"""Data path: the dataset statistics a DP model is built with and the batching of training
images, the GPU form of MatPL's loader side (src/pre_data/dpuni_data_loader.py,
src/PWMLFF/dp_mods/dp_trainer.py).

* ``set_davg_dstd`` picks images like ``UniDataset.set_davg_dstd`` (:180-215: a shuffled pass
  that takes each element from the first images containing it, for up to 10 rounds) and gets
  each picked image's statistics from ``image_stats``: the neighbor lists of
  ``matpl_neighbor_build`` and the per-type sums of the smoothed environment rows of
  ``matpl_env_stats`` (csrc/data.cu), turned into davg / dstd with the arithmetic of
  ``calc_stat`` (:422-499).  Images of one shape are searched together as a batch.
* ``set_energy_shift`` is ``UniDataset.set_energy_shift`` (:217-255): element counts against
  energies of a shuffled pass, least squares.
* ``classify_batches`` is ``_classify_batchs`` (dp_trainer.py:536-547): images grouped by their
  per-element atom counts; ``uniform_batches`` groups images of identical atom count and
  element sequence into [B, N] batches the fused kernels take in one launch.

Images are ``matpl_gb300.structures.Structure`` (types = indices into the model's atom_type
after ``model_types``).  The shuffles take a ``random.Random`` (the reference uses the global
one: seed it and pass ``random`` itself for the same picks).
"""
import random as _random
from collections import defaultdict
from typing import Dict, List, Sequence, Tuple

import numpy as np
import torch

from . import _lib, ops
from ._lib import check, ptr
from .params import DPConfig


def model_types(st, atom_type: Sequence[int]) -> np.ndarray:
    """Model type index of every atom (type_map of dpuni_data_loader.py:566-589)."""
    z = np.asarray(st.elements)[np.asarray(st.types)]
    at = list(atom_type)
    missing = set(z.tolist()) - set(at)
    if missing:
        raise _lib.MatplError(f"elements {sorted(missing)} are not in the model's atom_type")
    return np.array([at.index(int(v)) for v in z], dtype=np.int32)


@_lib.on_device
def image_stats(cfg: DPConfig, images: Sequence, device="cuda") -> List[Dict]:
    """Per image: {types: model types present (first-appearance order), counts, sums [T, 8]}
    with sums[t] = (sum Ri_0, sum Ri_0^2, sum Ri_x, sum Ri_x^2, ... Ri_z) over every slot of the
    atoms of type t (the neighbor search of calculate_davg_dstd, :377-420, with the model's m,
    Rc and per-type Rc)."""
    dev = torch.device(device)
    out: List[Dict] = [None] * len(images)
    groups: Dict[Tuple, List[int]] = defaultdict(list)
    tmaps = [model_types(st, cfg.atom_type) for st in images]
    for k, st in enumerate(images):
        groups[(st.natoms, tuple(tmaps[k].tolist()))].append(k)
    lib = _lib.load()
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    for (N, tm), idx in groups.items():
        tmap = torch.tensor(tm, dtype=torch.int32)
        frac = torch.tensor(np.stack([images[k].frac for k in idx]), device=dev)
        lat = torch.tensor(np.stack([images[k].lattice for k in idx]), device=dev)
        ln, idr = ops.find_neighbore(tmap, frac, lat, cfg.ntypes, cfg.maxNeighborNum, cfg.Rmax,
                                     cfg.Rmax)
        B = len(idx)
        sums = torch.empty(B, cfg.ntypes, 8, dtype=torch.float64, device=dev)
        tmd = tmap.to(dev)
        check(lib.matpl_env_stats(B, N, ln.shape[-1], cfg.ntypes, ptr(tmd), ptr(ln), ptr(idr),
                                  float(cfg.Rmin), float(cfg.Rmax), ptr(sums), ptr(err),
                                  torch.cuda.current_stream(dev).cuda_stream), "matpl_env_stats")
        s_h = sums.cpu().numpy()
        tm_np = np.asarray(tm)
        _, first, counts = np.unique(tm_np, return_index=True, return_counts=True)
        order = np.argsort(first)
        present = np.unique(tm_np)[order]
        for b, k in enumerate(idx):
            out[k] = {"types": present.tolist(), "counts": counts[order].tolist(), "sums": s_h[b]}
    if int(err.item()):
        raise _lib.MatplError("matpl_env_stats: atom type outside the model's types")
    return out


def _std(s2, s, n):
    # compute_std of calc_stat (dpuni_data_loader.py:423-429)
    if n == 0:
        return 1e-2
    v = np.sqrt(s2 / n - (s / n) * (s / n))
    return 1e-2 if np.abs(v) < 1e-2 else v


def stat_units(cfg: DPConfig, rec: Dict) -> Tuple[np.ndarray, np.ndarray]:
    """davg / dstd 4-vectors of each present type of one image (calc_stat, :459-490): the slot
    count of a type is its atoms x m x (number of present types), the angular channels use the
    mean of the three sums."""
    P = len(rec["types"])
    davg, dstd = [], []
    for t, n_at in zip(rec["types"], rec["counts"]):
        s = rec["sums"][t]
        n = n_at * cfg.maxNeighborNum * P
        sa, s2a = np.mean([s[2], s[4], s[6]]), np.mean([s[3], s[5], s[7]])
        davg.append([s[0] / (n + 1e-15), 0.0, 0.0, 0.0])
        dstd.append([_std(s[1], s[0], n), _std(s2a, sa, n), _std(s2a, sa, n), _std(s2a, sa, n)])
    return np.array(davg), np.array(dstd)


def set_davg_dstd(cfg: DPConfig, images: Sequence, rng=None, device="cuda", stats_fn=None
                  ) -> Tuple[np.ndarray, np.ndarray]:
    """davg, dstd [ntypes, ntypes * m * 4] (the model buffers), picking images like
    UniDataset.set_davg_dstd (:180-215).  ``stats_fn(cfg, images)`` replaces ``image_stats``
    (tests)."""
    rng = rng if rng is not None else _random
    shuffled = rng.sample(list(range(len(images))), len(images))
    S = cfg.ntypes * cfg.maxNeighborNum
    davg_d: Dict[int, list] = {t: [] for t in range(cfg.ntypes)}
    dstd_d: Dict[int, list] = {t: [] for t in range(cfg.ntypes)}
    searched, repeat = set(), 0
    picked = []
    for k in shuffled:                       # pass 1: which images the loop visits
        tm = model_types(images[k], cfg.atom_type)
        _, first = np.unique(tm, return_index=True)
        cout = np.unique(tm)[np.argsort(first)].tolist()
        picked.append((k, cout))
        for t in cout:
            searched.add(t)
        if len(searched) == cfg.ntypes:
            repeat += 1
            searched.clear()
        if repeat > 10:
            break
    sel = [images[k] for k, _ in picked]
    stats = stats_fn(cfg, sel) if stats_fn is not None else image_stats(cfg, sel, device=device)
    searched.clear()
    repeat = 0
    for (k, cout), rec in zip(picked, stats):  # pass 2: the reference's bookkeeping
        du, su = stat_units(cfg, rec)
        for i, t in enumerate(cout):
            if t not in searched:
                searched.add(t)
                davg_d[t].append(np.tile(du[i], S).reshape(-1, 4))
                dstd_d[t].append(np.tile(su[i], S).reshape(-1, 4))
        if len(searched) == cfg.ntypes:
            repeat += 1
            searched.clear()
        if repeat > 10:
            break
    davg = np.array([np.mean(np.array(davg_d[t]), axis=0).flatten() for t in range(cfg.ntypes)])
    dstd = np.array([np.mean(np.array(dstd_d[t]), axis=0).flatten() for t in range(cfg.ntypes)])
    return davg, dstd


def set_energy_shift(images: Sequence, energies: Sequence[float], atom_type: Sequence[int],
                     rng=None) -> np.ndarray:
    """Per-element energy shift: least squares of image energies against element counts over a
    shuffled pass (UniDataset.set_energy_shift, :217-255)."""
    rng = rng if rng is not None else _random
    order = rng.sample(list(range(len(images))), len(images))
    counts: Dict[int, list] = {z: [] for z in atom_type}
    E = []
    searched, repeat = set(), 0
    for k in order:
        z = np.asarray(images[k].elements)[np.asarray(images[k].types)]
        uz, cz = np.unique(z, return_counts=True)
        d = dict(zip(uz.tolist(), cz.tolist()))
        for el in atom_type:
            counts[el].append(d.get(el, 0))
        E.append(energies[k])
        searched.update(d.keys())
        if len(searched) == len(atom_type):
            repeat += 1
            searched.clear()
        if repeat > 5:
            break
    A = np.array([counts[el] for el in atom_type]).T
    x, *_ = np.linalg.lstsq(A, np.asarray(E), rcond=None)
    return np.array(x)


def classify_batches(type_maps: torch.Tensor, ntypes: int) -> List[List[int]]:
    """_classify_batchs (dp_trainer.py:536-547): indices of the images of a batch grouped by
    their per-type atom counts (type_maps [B, N], -1 = padding), in first-seen order."""
    groups: Dict[tuple, List[int]] = {}
    for b, row in enumerate(type_maps.cpu()):
        key = tuple(torch.bincount(row[row != -1].long(), minlength=ntypes).tolist())
        groups.setdefault(key, []).append(b)
    return list(groups.values())


def uniform_batches(images: Sequence, atom_type: Sequence[int],
                    max_batch: int = 64) -> List[List[int]]:
    """Images of identical atom count and element sequence, at most ``max_batch`` per group:
    each group is one [B, N] launch of the fused kernels (uneven datasets need no padding)."""
    groups: Dict[tuple, List[int]] = {}
    for k, st in enumerate(images):
        key = (st.natoms, tuple(model_types(st, atom_type).tolist()))
        groups.setdefault(key, []).append(k)
    out = []
    for idx in groups.values():
        for a in range(0, len(idx), max_batch):
            out.append(idx[a:a + max_batch])
    return out


@_lib.on_device
def ragged_batch(cfg: DPConfig, images: Sequence, device="cuda", energies=None, forces=None,
                 out_dtype: torch.dtype = torch.float64) -> Dict:
    """Ragged collate: configurations of uneven atom count and composition concatenated into
    one image of sum(N_c) atoms, the training batch of ``FusedTrainer`` / ``GraphedTrainer``
    without ``_classify_batchs``' per-composition clusters (dp_trainer.py:536-547).

    Each configuration's neighbor list comes from ``matpl_neighbor_build`` on its own cell
    (``find_neighbore``, dpuni_data_loader.py:595-650) and its neighbor indices are shifted by
    the configuration's first atom, so no pair crosses configurations; the per-atom quantities
    of the fused kernels then need no padding, and energies are per-configuration sums of the
    atoms' energies (``config_of_atom``).  Returns a batch dict: list_neigh [1, sum N, S] int32
    (1-based, 0 = empty), ImageDR [1, sum N, S, 4], type_map [sum N], atom_type,
    config_of_atom [sum N] int64, natoms [C] int64, and, when given, Etot [C] and Force
    [1, sum N, 3] labels."""
    dev = torch.device(device)
    S = cfg.ntypes * cfg.maxNeighborNum
    lns, idrs, tms, cfg_of = [], [], [], []
    start = 0
    for c, st in enumerate(images):
        tm = torch.tensor(model_types(st, cfg.atom_type), device=dev)
        ln, idr = ops.find_neighbore(tm, torch.tensor(st.frac, device=dev),
                                     torch.tensor(st.lattice, device=dev), cfg.ntypes,
                                     cfg.maxNeighborNum, float(cfg.Rmax), float(cfg.Rmax),
                                     out_dtype=out_dtype)
        lns.append(torch.where(ln > 0, ln + start, ln))
        idrs.append(idr)
        tms.append(tm)
        cfg_of.append(torch.full((st.natoms,), c, dtype=torch.int64, device=dev))
        start += st.natoms
    batch = {"list_neigh": torch.cat(lns, 1).contiguous(),
             "ImageDR": torch.cat(idrs, 1).contiguous(),
             "type_map": torch.cat(tms).to(torch.int32).contiguous(),
             "atom_type": list(cfg.atom_type),
             "config_of_atom": torch.cat(cfg_of).contiguous(),
             "natoms": torch.tensor([st.natoms for st in images], dtype=torch.int64, device=dev)}
    assert batch["list_neigh"].shape == (1, start, S)
    if energies is not None:
        batch["Etot"] = torch.as_tensor(energies, dtype=torch.float64).to(dev).reshape(-1)
    if forces is not None:
        batch["Force"] = torch.cat([torch.as_tensor(f, dtype=torch.float64).to(dev).reshape(-1, 3)
                                    for f in forces]).reshape(1, start, 3)
    return batch


def config_energies(Ei_atom: torch.Tensor, config_of_atom: torch.Tensor, nconfig: int) -> torch.Tensor:
    """Per-configuration energy of a ragged batch: the sum of its atoms' energies."""
    out = torch.zeros(nconfig, dtype=Ei_atom.dtype, device=Ei_atom.device)
    return out.index_add(0, config_of_atom, Ei_atom.reshape(-1))
