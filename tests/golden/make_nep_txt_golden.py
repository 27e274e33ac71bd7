"""Generate the nep5 potential-file fixtures by running MatPL's own converter.

Runs only where the MatPL source tree is mounted (path in MATPL_REF, default: a ``reference``
directory beside the repository root); the committed ``nep_txt_*.txt`` files are what the tests
read.  For each case it builds seeded parameters with ``matpl_gb300.nep.init_params`` (the
reference's shapes), a q_scaler, and a checkpoint dictionary with the keys the reference's
converter reads (``json_file`` with model_type / atom_type / descriptor / fitting_net,
``state_dict``, ``q_scaler``, ``max_neighbor``), saves it with ``torch.save`` into a temporary
directory, and runs ``extract_model`` of utils/nep_to_gpumd.py on it; the text it returns is the
fixture.

Usage:  python tests/golden/make_nep_txt_golden.py
"""
import importlib.util
import os
import sys
import tempfile

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from matpl_gb300 import nep as NP  # noqa: E402
from oracle.refpath import reference_root  # noqa: E402

# name: (elements, n_max, basis_size, l_max, neuron, zbl, max_neighbor, seed)
CASES = {
    "hfo_l4": ([8, 72], (4, 4), (5, 5), (4, 2, 1), 10, None, (90, 40), 3),
    "q4_zbl": ([3, 14, 8, 72], (3, 2), (4, 3), (3, 1, 0), 6, 2.0, (120, 60), 4),
    "si_2b": ([14], (5, 3), (6, 4), (0, 0, 0), 8, None, (70, 20), 5),
}


def case_params(name):
    el, n_max, basis, l_max, neuron, zbl, mx, seed = CASES[name]
    cfg = NP.NepConfig(atom_type=el, cutoff=(6.0, 4.0), n_max=n_max, basis_size=basis,
                       l_max=l_max, neuron=neuron, zbl=zbl)
    prm = NP.init_params(cfg, seed, energy_shift=-2.5)
    g = torch.Generator().manual_seed(seed + 50)
    prm["q_scaler"] = 0.5 + torch.rand(cfg.feature_nums, generator=g, dtype=torch.float64)
    if cfg.l_max[0] == 0:
        prm.pop("c_param_3", None)
    return cfg, prm, mx


def main():
    path = os.path.join(reference_root(), "utils", "nep_to_gpumd.py")
    spec = importlib.util.spec_from_file_location("ref_nep_to_gpumd", path)
    conv = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(conv)
    for name in CASES:
        cfg, prm, mx = case_params(name)
        desc = {"Rmax": cfg.cutoff[0], "Rmin": 0.5, "cutoff": list(cfg.cutoff),
                "n_max": list(cfg.n_max), "basis_size": list(cfg.basis_size),
                "l_max": list(cfg.l_max), "type_weight": [1.0] * cfg.ntypes}
        if cfg.zbl is not None:
            desc["zbl"] = cfg.zbl
        ckpt = {"json_file": {"model_type": "NEP", "atom_type": list(cfg.atom_type),
                              "model": {"descriptor": desc,
                                        "fitting_net": {"network_size": [cfg.neuron, 1]}}},
                "state_dict": {k: v for k, v in prm.items() if k != "q_scaler"},
                "q_scaler": [float(x) for x in prm["q_scaler"]],
                "max_neighbor": list(mx), "epoch": 1}
        with tempfile.TemporaryDirectory() as d:
            p = os.path.join(d, "nep_model.ckpt")
            torch.save(ckpt, p)
            text, _, _ = conv.extract_model(p)
        out = os.path.join(HERE, f"nep_txt_{name}.txt")
        with open(out, "w") as f:
            f.write(text)
        print(out, len(text.splitlines()), "lines")


if __name__ == "__main__":
    main()
