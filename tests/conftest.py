import os
import sys

import numpy as np
import pytest
import torch

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz"), allow_pickle=False))


class GoldenCase:
    """Rebuilds the inputs of a golden fixture: structure, oracle neighbor list, weights."""

    def __init__(self, name):
        from matpl_gb300 import params as P
        from oracle import neigh
        g = load_golden(name)
        self.g = g
        self.name = name
        self.dtype = torch.float64 if str(g["dtype"]) == "float64" else torch.float32
        self.cfg = P.DPConfig(atom_type=[int(x) for x in g["atom_type"]], maxNeighborNum=int(g["m"]),
                              Rmax=float(g["Rmax"]), Rmin=float(g["Rmin"]))
        lat, frac, types = g["lattice"], g["frac"], g["types"]
        lns, idrs = [], []
        for b in range(lat.shape[0]):
            ln, idr = neigh.find_neighbore(types, frac[b], lat[b], self.cfg.ntypes,
                                           self.cfg.maxNeighborNum, self.cfg.Rmax,
                                           [self.cfg.Rmax] * self.cfg.ntypes)
            lns.append(ln[0]); idrs.append(idr[0])
        self.list_neigh = np.stack(lns)
        self.image_dr = np.stack(idrs)
        self.types = types.astype(np.int32)
        if "seed_w" in g:
            self.params = P.init_params(self.cfg, int(g["seed_w"]))
        else:
            self.params = {k[2:]: torch.tensor(v) for k, v in g.items() if k.startswith("w:")}
            self.params = P.load_reference_state_dict(self.params)
        self.davg = torch.tensor(g["davg"])
        self.dstd = torch.tensor(g["dstd"])


@pytest.fixture(scope="session")
def golden_case():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = GoldenCase(name)
        return cache[name]
    return get


class NepCase:
    """Rebuilds the inputs of a NEP golden fixture: frames, oracle neighbor lists, parameters
    (seeded, with the fixture's q_scaler)."""

    def __init__(self, name):
        from matpl_gb300 import nep as NP
        from oracle import nep_oracle as NO
        g = load_golden(name)
        self.g = g
        self.name = name
        self.cfg = NP.NepConfig(atom_type=[int(x) for x in g["atom_type"]],
                                cutoff=tuple(float(x) for x in g["cutoff"]),
                                n_max=tuple(int(x) for x in g["n_max"]),
                                basis_size=tuple(int(x) for x in g["basis_size"]),
                                l_max=tuple(int(x) for x in g["l_max"]),
                                neuron=int(g["neuron"]), train_2b=bool(g["train_2b"]),
                                zbl=(float(g["zbl"]) if "zbl" in g and not np.isnan(g["zbl"])
                                     else None))
        self.frames = NP.NepFrames(g["position"].copy(), g["type_map"], g["num_atom"], g["box"],
                                   g["box_orig"], g["num_cell"])
        self.params = NP.init_params(self.cfg, int(g["seed_w"]), energy_shift=-3.0)
        self.params["q_scaler"] = torch.tensor(g["q_scaler"])
        (self.NN_r, self.NN_a, self.NL_r, self.NL_a, self.Ri_r,
         self.Ri_a) = NO.neighbor(self.frames, self.cfg.cutoff[0], self.cfg.cutoff[1],
                                  int(g["max_r"]), int(g["max_a"]))


@pytest.fixture(scope="session")
def nep_case():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = NepCase(name)
        return cache[name]
    return get
