"""Autotuner for the tile shape of the mixed-precision (tcgen05) embedding kernels.

The mixed kernels walk the occupied neighbor slots of a group of centre atoms in 128-row tensor
core tiles, one tile per embedding net at a time.  The group size decides how full those tiles
are (about group_atoms * neighbors / ntypes^2 rows per net and group) and, with the CTAs per SM,
how much latency of the MMA round trips the SM can hide.  The best pair depends on the neighbor
density, the number of types and the batch, so it is measured: every candidate is set through
``matpl_dp_set_tuning`` and timed with CUDA events on the caller's own evaluation; the fastest
stays set.  Results do not depend on the choice (the per-atom arithmetic is the same), which
``tune_dp_mixed`` checks on the candidates' outputs as it goes.
"""
import ctypes
import json
import os
from typing import Dict, Iterable, Optional, Sequence, Tuple

import torch

from . import _lib
from ._lib import check

DEFAULT_GROUPS = (6, 8, 10, 11, 12, 14, 16)
DEFAULT_CTAS = (2, 3, 4)


def set_tuning(group_atoms: int = 0, ctas_per_sm: int = 0):
    check(_lib.load().matpl_dp_set_tuning(int(group_atoms), int(ctas_per_sm)),
          "matpl_dp_set_tuning")


def get_tuning() -> Tuple[int, int]:
    a, b = ctypes.c_int(), ctypes.c_int()
    check(_lib.load().matpl_dp_get_tuning(ctypes.byref(a), ctypes.byref(b)), "matpl_dp_get_tuning")
    return a.value, b.value


def _key(model, list_neigh, present) -> str:
    B, N, S = list_neigh.shape
    return f"{model.precision}:B{B}:N{N}:S{S}:T{model.cfg.ntypes}:P{''.join(map(str, present))}"


def tune_dp_mixed(model, list_neigh: torch.Tensor, type_map: torch.Tensor, present: Sequence[int],
                  image_dr: torch.Tensor, groups: Iterable[int] = DEFAULT_GROUPS,
                  ctas: Iterable[int] = DEFAULT_CTAS, reps: int = 5,
                  cache_path: Optional[str] = None,
                  num_neigh: Optional[torch.Tensor] = None) -> Dict:
    """Time ``model.evaluate`` (a ``matpl_gb300.dp.DP`` in a mixed form) for every
    (group_atoms, ctas_per_sm) candidate, keep the fastest set and return the table.
    ``cache_path``: optional JSON file of earlier results keyed by precision, batch shape and
    types; a hit sets the stored choice without timing.  ``num_neigh``: block lengths of an
    occupied-slot list (``find_neighbore(..., occupied_only=True)``)."""
    if not model.precision.startswith("mixed"):
        raise _lib.MatplError("only the mixed forms have tunable tiles")
    key = _key(model, list_neigh, present)
    cache = {}
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            cache = json.load(f)
        if key in cache:
            set_tuning(cache[key]["group_atoms"], cache[key]["ctas_per_sm"])
            return dict(cache[key], cached=True)
    ref = None
    table = []
    best = None
    for g in groups:
        for c in ctas:
            set_tuning(g, c)
            for _ in range(2):
                r = model.evaluate(list_neigh, type_map, present, image_dr, 0, num_neigh=num_neigh)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                r = model.evaluate(list_neigh, type_map, present, image_dr, 0, num_neigh=num_neigh)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            if ref is None:
                ref = r["Force"].clone()
            else:
                dev = (r["Force"] - ref).abs().max().item()
                scale = ref.abs().max().item() + 1e-30
                if dev > 1e-4 * scale:
                    set_tuning(0, 0)
                    raise _lib.MatplError(f"tile shape ({g}, {c}) changed the forces by {dev}")
            table.append({"group_atoms": g, "ctas_per_sm": c, "ms": ms})
            if best is None or ms < best["ms"]:
                best = table[-1]
    set_tuning(best["group_atoms"], best["ctas_per_sm"])
    result = {"group_atoms": best["group_atoms"], "ctas_per_sm": best["ctas_per_sm"],
              "ms": best["ms"], "table": table, "cached": False}
    if cache_path:
        cache[key] = {k: result[k] for k in ("group_atoms", "ctas_per_sm", "ms")}
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    return result
