"""Generate the golden fixtures of the NEP training derivatives from MatPL's own NEP code.

Runs only where the MatPL source tree is mounted (path in MATPL_REF, default: a
``reference`` directory beside the repository root);
the committed ``nep_train_*.npz`` files are what the tests read.  For two of the NEP cases
(``nep_q4_tri2``: four elements, two triclinic frames, l_max 4/2/1; ``nep_hfo_l4``: two
elements, 3-body only) it rebuilds the inputs exactly as ``make_nep_golden.py`` does (the
reference's CPU neighbor operator, seeded parameters, the fixture's q_scaler) and runs the
reference ``src.model.nep_net.NEP`` CPU branch under autograd:

1. descriptor derivatives, the quantities CalcOps calculateNepFeat / calculateNepMbFeat and
   their Grad functions return (src/op/src/CalcOps.cpp:385-1023): for a seeded G = dL/dq the
   first backward dL/dc2, dL/dc3, dL/dRi_radial, dL/dRi_angular of L = sum G * calculate_qn, and
   for seeded H_r, H_a the second backward (gradients of sum H * dL/dRi with respect to G, c2,
   c3);
2. the training gradient: every parameter's gradient of
   L = sum gE * Etot + sum gF * Force + sum gV * Virial through ``NEP.forward`` (create_graph
   forces, as loss.backward() sees it in nep_trainer.py) for seeded gE, gF, gV.

Seeds (numpy default_rng) and shapes are stored, so tests regenerate G, H, gE, gF, gV.

Usage:  python tests/golden/make_nep_train_golden.py
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from matpl_gb300 import nep as NP  # noqa: E402
from make_nep_golden import fake_input_param, reference_nep_class  # noqa: E402

CASES = {"nep_q4_tri2": 402, "nep_hfo_l4": 403}


def seeded(seed, shape):
    return np.random.default_rng(seed).standard_normal(shape)


def cfg_of(g):
    return NP.NepConfig(atom_type=[int(a) for a in g["atom_type"]],
                        cutoff=tuple(float(c) for c in g["cutoff"]),
                        n_max=tuple(int(v) for v in g["n_max"]),
                        basis_size=tuple(int(v) for v in g["basis_size"]),
                        l_max=tuple(int(v) for v in g["l_max"]), neuron=int(g["neuron"]),
                        train_2b=bool(g["train_2b"]))


def run(name, seed_w, NEP, ops):
    g = dict(np.load(os.path.join(HERE, f"{name}.npz")))
    cfg = cfg_of(g)
    t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt)  # noqa: E731
    num_atom = t(g["num_atom"].reshape(-1, 1), torch.int64)
    tmap = t(g["type_map"], torch.int64)
    ftype = t(np.arange(cfg.ntypes), torch.int64)
    NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = ops.calculate_neighbor(
        num_atom, tmap, ftype, t(g["box"], torch.float64), t(g["box_orig"], torch.float64),
        t(g["num_cell"], torch.int64), t(g["position"], torch.float64), cfg.cutoff[0],
        cfg.cutoff[1], int(g["max_r"]), int(g["max_a"]), True)
    model = NEP(fake_input_param(cfg), [0.0] * cfg.ntypes).to(torch.float64)
    p = NP.init_params(cfg, seed_w, energy_shift=-3.0)
    with torch.no_grad():
        model.c_param_2.copy_(p["c_param_2"])
        if cfg.l_max[0] > 0:
            model.c_param_3.copy_(p["c_param_3"])
        for ty in range(cfg.ntypes):
            for li in range(2):
                pre = f"fitting_net.{ty}.layers.{li}."
                model.fitting_net[ty].layers[li].weight.copy_(p[pre + "weight"])
                model.fitting_net[ty].layers[li].bias.copy_(p[pre + "bias"])
    model.set_nep_param_device(q_scaler=g["q_scaler"])
    model.reset_scaler(g["q_scaler"], torch.float64, "cpu")
    N = int(tmap.shape[0])
    F = cfg.feature_nums
    rec = {"name": name, "seed_w": seed_w, "seed_G": 11, "seed_Hr": 12, "seed_Ha": 13,
           "seed_gE": 14, "seed_gF": 15, "seed_gV": 16}

    # 1. descriptor derivatives through calculate_qn
    jt_r = torch.where(NL_r >= 0, tmap[NL_r.clamp(min=0)], torch.full_like(NL_r, -1))
    jt_a = torch.where(NL_a >= 0, tmap[NL_a.clamp(min=0)], torch.full_like(NL_a, -1))
    Rr = Ri_r.clone().requires_grad_()
    Ra = Ri_a.clone().requires_grad_()
    feats = model.calculate_qn(tmap, jt_r.clone(), Rr, jt_a.clone(), Ra, torch.device("cpu"),
                               torch.float64)
    G = torch.tensor(seeded(rec["seed_G"], (N, F))).requires_grad_()
    params = [model.c_param_2] + ([model.c_param_3] if cfg.l_max[0] > 0 else [])
    first = torch.autograd.grad((feats * G).sum(), params + [Rr, Ra], create_graph=True,
                                allow_unused=True)
    gc2, gc3 = first[0], first[1] if cfg.l_max[0] > 0 else None
    gRr, gRa = first[len(params)], first[len(params) + 1]
    Hr = torch.tensor(seeded(rec["seed_Hr"], tuple(Ri_r.shape)))
    Ha = torch.tensor(seeded(rec["seed_Ha"], tuple(Ri_a.shape)))
    second = torch.autograd.grad((gRr * Hr).sum() + (gRa * Ha).sum(), [G] + params,
                                 allow_unused=True)
    rec.update(first_c2=gc2.detach().numpy(), first_Rr=gRr.detach().numpy(),
               first_Ra=gRa.detach().numpy(), second_G=second[0].numpy(),
               second_c2=second[1].numpy())
    if cfg.l_max[0] > 0:
        rec.update(first_c3=gc3.detach().numpy(), second_c3=second[2].numpy())

    # 2. the training gradient through NEP.forward
    model.zero_grad(set_to_none=True)
    Etot, Ei, Force, _, Virial = model(NN_r.clone(), NL_r.clone(), Ri_r.clone(), NN_a.clone(),
                                       NL_a.clone(), Ri_a.clone(), num_atom, tmap)
    B = Etot.shape[0]
    gE = torch.tensor(seeded(rec["seed_gE"], (B,)))
    gF = torch.tensor(seeded(rec["seed_gF"], (N, 3)))
    gV = torch.tensor(seeded(rec["seed_gV"], (B, 9)))
    L = (gE * Etot.reshape(-1)).sum() + (gF * Force).sum() + (gV * Virial).sum()
    L.backward()
    for k, v in model.named_parameters():
        if v.grad is not None:
            rec["train:" + k] = v.grad.detach().numpy()
    rec.update(train_Etot=Etot.detach().numpy(), train_Force=Force.detach().numpy(),
               train_Virial=Virial.detach().numpy())
    np.savez_compressed(os.path.join(HERE, f"nep_train_{name[4:]}.npz"), **rec)
    print(name, "N", N, "F", F, "|dc2|", float(gc2.abs().max()), "|train c2|",
          float(model.c_param_2.grad.abs().max()))


def main():
    NEP, ops = reference_nep_class()
    for name, seed_w in CASES.items():
        run(name, seed_w, NEP, ops)


if __name__ == "__main__":
    main()
