"""Generate the golden fixture of the type-embedding DP model from MatPL's own code.

Runs only where the MatPL source tree is mounted (path in MATPL_REF, default: a
``reference`` directory beside the repository root);
the committed ``typedp_hfo48.npz`` is what the tests read.  On the ``hfo48_f64`` structure
(HfO2, 48 atoms; its davg / dstd) it builds the reference ``src.model.dp_dp_typ_emb.TypeDP``
(CPU branch) with seeded parameters (``matpl_gb300.typedp.init_type_params``) and three physical
properties, evaluates E, Ei, F, V, and the parameter gradient of a seeded E + F loss (force
term through create_graph, as training sees it).  The element vectors the reference derives
from its property table are stored with the outputs.

Usage:  python tests/golden/make_typedp_golden.py
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from matpl_gb300 import params as P  # noqa: E402
from matpl_gb300.typedp import init_type_params  # noqa: E402
from make_golden import ref_config  # noqa: E402
from oracle import neigh  # noqa: E402

from oracle.refpath import reference_root  # noqa: E402

REF = reference_root()
PROPS = ["atomic_number", "atom_mass", "atom_radius"]
SEED_W = 611


def main():
    sys.path.insert(0, REF)
    sys.path.insert(0, os.path.join(REF, "src"))
    real = torch.ops.load_library
    torch.ops.load_library = lambda path: None
    try:
        from src.model.dp_dp_typ_emb import TypeDP
    finally:
        torch.ops.load_library = real
    g = dict(np.load(os.path.join(HERE, "hfo48_f64.npz")))
    cfg = P.DPConfig(atom_type=[int(a) for a in g["atom_type"]], maxNeighborNum=int(g["m"]),
                     Rmax=float(g["Rmax"]), Rmin=float(g["Rmin"]))
    conf = ref_config(cfg, "float64")
    conf["net_cfg"]["type_embedding_net"] = {"network_size": [], "bias": True,
                                             "resnet_dt": False, "activation": "tanh",
                                             "physical_property": PROPS}
    model = TypeDP(conf, g["davg"], g["dstd"], [0.0] * cfg.ntypes).to(torch.float64)
    sd = init_type_params(cfg, len(PROPS), SEED_W)
    msd = model.state_dict()
    assert set(msd) == set(sd), (sorted(msd), sorted(sd))
    model.load_state_dict(sd)
    types_ = g["types"].astype(np.int32)
    ln, idr = neigh.find_neighbore(types_, g["frac"][0], g["lattice"][0], cfg.ntypes,
                                   cfg.maxNeighborNum, cfg.Rmax, [cfg.Rmax] * cfg.ntypes)
    at = torch.tensor(cfg.atom_type, dtype=torch.int32)
    Etot, Ei, F, _, V = model(torch.tensor(ln, dtype=torch.int32),
                              torch.tensor(types_, dtype=torch.int32), at,
                              torch.tensor(idr, dtype=torch.float64), 0)
    rng = np.random.default_rng(17)
    gE = rng.standard_normal(1)
    gF = rng.standard_normal(tuple(F.shape))
    L = (torch.tensor(gE) * Etot.reshape(-1)).sum() + (torch.tensor(gF) * F).sum()
    L.backward()
    rec = {"props": np.array(PROPS), "seed_w": SEED_W, "seed_g": 17,
           "type_vector": np.array([model.type_vector[z] for z in cfg.atom_type]),
           "Etot": Etot.detach().numpy(), "Ei": Ei.detach().numpy(), "Force": F.detach().numpy(),
           "Virial": V.detach().numpy()}
    for k, v in model.named_parameters():
        rec["grad:" + k] = v.grad.numpy()
    np.savez_compressed(os.path.join(HERE, "typedp_hfo48.npz"), **rec)
    print("E", Etot.item(), "max|F|", F.abs().max().item(), "vectors", rec["type_vector"])


if __name__ == "__main__":
    main()
