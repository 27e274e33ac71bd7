"""Generate the golden fixture of the compressed DP model from MatPL's own code.

Runs only where the MatPL source tree is mounted (path in MATPL_REF, default: a
``reference`` directory beside the repository root);
the committed ``compress_*.npz`` files are what the tests read.  For a seeded two-element DP
(the ``hfo48_f64`` case: its structure, weights, davg / dstd) it builds the compression table
with the reference's own ``set_sij_range`` and ``dp_model_compress_5order`` /
``dp_model_compress_3order`` (src/user/ckpt_compress.py; the modules it imports for its command
line are stood in for) on the reference ``dp_dp_script.DP``, installs it with ``set_comp_tab``
and evaluates the model (the compress branch of calculate_xyz_scater on CPU).  Stored: the
table's shape, checksum and a sample of rows, and E, Ei, F, V.

Usage:  python tests/golden/make_compress_golden.py
"""
import hashlib
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from matpl_gb300 import params as P  # noqa: E402
from make_golden import ref_config  # noqa: E402
from oracle import neigh  # noqa: E402

from oracle.refpath import reference_root  # noqa: E402

REF = reference_root()
DX = 0.02
SIJ_MAX_PAD = 1.0   # raw s maximum of the "training data": the case's own maximum times this


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load_reference():
    for name in ("src.user.input_param", "src.PWMLFF", "src.PWMLFF.dp_network",
                 "src.model.dp_dp", "src.model.dp_dp_typ_emb", "utils",
                 "utils.atom_type_emb_dict"):
        sys.modules[name] = types.ModuleType(name)
    sys.modules["src.user.input_param"].InputParam = object
    sys.modules["src.PWMLFF.dp_network"].dp_network = object
    sys.modules["src.model.dp_dp"].DP = object
    sys.modules["src.model.dp_dp_typ_emb"].TypeDP = object
    sys.modules["utils.atom_type_emb_dict"].get_normalized_data_list = None
    sys.path.insert(0, REF)
    sys.path.insert(0, os.path.join(REF, "src"))
    from src.user import ckpt_compress as cc
    from src.model.dp_dp_script import DP
    return cc, DP


def main():
    cc, DP = load_reference()
    g = dict(np.load(os.path.join(HERE, "hfo48_f64.npz")))
    cfg = P.DPConfig(atom_type=[int(a) for a in g["atom_type"]], maxNeighborNum=int(g["m"]),
                     Rmax=float(g["Rmax"]), Rmin=float(g["Rmin"]))
    types_ = g["types"].astype(np.int32)
    ln, idr = neigh.find_neighbore(types_, g["frac"][0], g["lattice"][0], cfg.ntypes,
                                   cfg.maxNeighborNum, cfg.Rmax, [cfg.Rmax] * cfg.ntypes)
    sd = P.init_params(cfg, int(g["seed_w"]))
    davg, dstd = g["davg"], g["dstd"]
    model = DP(ref_config(cfg, "float64"), davg, dstd, [0.0] * cfg.ntypes).to(torch.float64)
    model.load_state_dict({k: sd[k].to(torch.float64) for k in model.state_dict()})
    # the largest raw s of the case (before davg / dstd), as training would record it
    r = idr[..., 0][ln > 0]
    u = (r - cfg.Rmin) / (cfg.Rmax - cfg.Rmin)
    vv = np.where(r < cfg.Rmin, 1.0, np.where(r < cfg.Rmax, u ** 3 * (-6 * u * u + 15 * u - 10) + 1,
                                              0.0))
    sij_max = float((vv / r).max()) * SIJ_MAX_PAD
    rec = {"sij_max_raw": sij_max, "dx": DX}
    for order in (5, 3):
        sij, smin, smax, out_max, len_sij, len_out = cc.set_sij_range(
            davg, dstd, cfg.atom_type, torch.float64, "cpu", sij_max, DX)
        fn = cc.dp_model_compress_5order if order == 5 else cc.dp_model_compress_3order
        tab = fn(sij, model, DX, len_sij, len_out)
        comp = {"table": tab, "dx": DX, "order": order, "sij_min": smin, "sij_max": smax,
                "sij_out_max": out_max, "sij_len": len_sij, "sij_out_len": len_out}
        model.set_comp_tab(comp)
        at = torch.tensor(cfg.atom_type, dtype=torch.int32)
        Etot, Ei, F, _, V = model(torch.tensor(ln, dtype=torch.int32),
                                  torch.tensor(types_, dtype=torch.int32), at,
                                  torch.tensor(idr, dtype=torch.float64), 0)
        rows = np.linspace(0, tab.shape[1] - 1, 7).astype(int)
        rec.update({f"o{order}_shape": np.array(tab.shape), f"o{order}_sha": sha(tab),
                    f"o{order}_rows": rows, f"o{order}_sample": tab[:, rows],
                    f"o{order}_grid": np.array([smin, smax, out_max, len_sij, len_out]),
                    f"o{order}_Etot": Etot.detach().numpy(), f"o{order}_Ei": Ei.detach().numpy(),
                    f"o{order}_Force": F.detach().numpy(), f"o{order}_Virial": V.detach().numpy()})
        model.compress_tab = None
        print("order", order, "table", tab.shape, "E", Etot.item())
    np.savez_compressed(os.path.join(HERE, "compress_hfo48.npz"), **rec)


if __name__ == "__main__":
    main()
