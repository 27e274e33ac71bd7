"""Generate the golden E/F/V fixtures by running MatPL's own DP implementation.

Runs only in a container where the MatPL source tree is mounted (path in MATPL_REF, default: a
``reference`` directory beside the repository root); the committed ``*.npz`` files are what the tests read.  For each case it

1. builds a seeded synthetic structure (``matpl_gb300.structures``),
2. builds the neighbor list with the oracle restatement of NeighConst.f90 (the Fortran module
   itself cannot be compiled without ifort),
3. sets davg/dstd with ``matpl_gb300.params.calc_stat`` and seeded weights,
4. evaluates the reference ``src.model.dp_dp_script.DP`` (pure-torch CPU path, the one MatPL
   exports to LAMMPS) and, for the real-weight case, the shipped TorchScript model
   ``src/lmps/lammps-libtorch/dp_lmps_demo/jit_dp.pt`` on its ``lmp.config``,
5. stores inputs that are cheap to rebuild (seeds, structure) plus the outputs and checksums.

Usage:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from matpl_gb300 import structures, params as P  # noqa: E402
from oracle import neigh  # noqa: E402

from oracle.refpath import reference_root  # noqa: E402

REF = reference_root()


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_config(cfg: P.DPConfig, dtype: str):
    return {
        "model_type": "DP",
        "atomType": [{"type": t, "Rc": cfg.Rmax, "Rm": cfg.Rmin} for t in cfg.atom_type],
        "M2": cfg.M2, "Rc_M": cfg.Rmax, "maxNeighborNum": cfg.maxNeighborNum,
        "training_type": dtype,
        "net_cfg": {
            "embedding_net": {"network_size": cfg.emb_sizes, "bias": True,
                              "resnet_dt": cfg.emb_resnet_dt, "activation": "tanh"},
            "fitting_net": {"network_size": cfg.fit_sizes, "bias": True,
                            "resnet_dt": cfg.fit_resnet_dt, "activation": "tanh"},
        },
    }


def run_reference_dp(cfg, sd, davg, dstd, ln, idr, tmap, dtype):
    sys.path.insert(0, REF)
    from src.model.dp_dp_script import DP  # the reference implementation
    tdt = torch.float64 if dtype == "float64" else torch.float32
    model = DP(ref_config(cfg, dtype), davg, dstd, [0.0] * cfg.ntypes).to(tdt)
    msd = model.state_dict()
    assert set(msd) == set(sd)
    model.load_state_dict({k: sd[k].to(tdt) for k in msd})
    ln_t = torch.tensor(ln, dtype=torch.int32)
    idr_t = torch.tensor(idr, dtype=tdt)
    tm = torch.tensor(tmap, dtype=torch.int32)
    at = torch.tensor(cfg.atom_type, dtype=torch.int32)
    Etot, Ei, F, _, V = model(ln_t, tm, at, idr_t, 0)
    # dE/dRi, as calculate_force_virial obtains it (dp_dp.py:429)
    B, N, S = ln_t.shape
    emb_list, type_nums = model.get_train_2body_type(at)
    Ri, Ri_d = model.calculate_Ri(N, B, S, tm, idr_t, idr_t.device, tdt)
    Ri.requires_grad_()
    Ei2 = model.calculate_Ei(tm, Ri, B, emb_list, type_nums, idr_t.device)
    dE = torch.autograd.grad([Ei2.sum(1)], [Ri], grad_outputs=[torch.ones(B, 1, dtype=tdt)])[0]
    return {k: v.detach().numpy() for k, v in
            dict(Etot=Etot, Ei=Ei, Force=F, Virial=V, dE=dE, Ri_d=Ri_d).items()}


def seeded_case(name, st, cfg, seed_w, dtype, keep_dE=False, batch_structs=None):
    structs = [st] + (batch_structs or [])
    lns, idrs = [], []
    for s in structs:
        ln, idr = neigh.find_neighbore(s.types, s.frac, s.lattice, cfg.ntypes,
                                       cfg.maxNeighborNum, cfg.Rmax, [cfg.Rmax] * cfg.ntypes)
        lns.append(ln[0]); idrs.append(idr[0])
    ln = np.stack(lns); idr = np.stack(idrs)
    davg, dstd = P.calc_stat(cfg, ln[:1], idr[:1], st.types)
    sd = P.init_params(cfg, seed_w)
    out = run_reference_dp(cfg, sd, davg, dstd, ln, idr, st.types, dtype)
    rec = dict(
        name=name, dtype=dtype, seed_w=seed_w,
        lattice=np.stack([s.lattice for s in structs]), frac=np.stack([s.frac for s in structs]),
        types=st.types, atom_type=np.array(cfg.atom_type), m=cfg.maxNeighborNum,
        Rmax=cfg.Rmax, Rmin=cfg.Rmin, davg=davg, dstd=dstd,
        list_sha=sha(ln), imagedr_sha=sha(idr), nneigh=(ln > 0).sum(-1).astype(np.int32),
        Etot=out["Etot"], Ei=out["Ei"], Force=out["Force"], Virial=out["Virial"],
        param_sha=sha(np.concatenate([v.numpy().ravel() for v in sd.values()])),
    )
    if keep_dE:
        rec["dE"] = out["dE"]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "E", out["Etot"].ravel()[:2], "max|F|", np.abs(out["Force"]).max(),
          "nneigh max", rec["nneigh"].max())


def jit_case():
    demo = os.path.join(REF, "src/lmps/lammps-libtorch/dp_lmps_demo")
    model = torch.jit.load(os.path.join(demo, "jit_dp.pt"))
    lines = open(os.path.join(demo, "lmp.config")).read().splitlines()
    nat = int([l for l in lines if l.strip().endswith("atoms")][0].split()[0])
    lo_hi = [list(map(float, [l for l in lines if l.strip().endswith(f"{a}lo {a}hi")][0]
                           .split()[:2])) for a in "xyz"]
    xy, xz, yz = map(float, [l for l in lines if l.strip().endswith("xy xz yz")][0].split()[:3])
    lat = np.array([[lo_hi[0][1] - lo_hi[0][0], 0, 0], [xy, lo_hi[1][1] - lo_hi[1][0], 0],
                    [xz, yz, lo_hi[2][1] - lo_hi[2][0]]])
    start = [i for i, l in enumerate(lines) if l.strip().startswith("Atoms")][0] + 2
    rows = [l.split() for l in lines[start:start + nat]]
    ltype = np.array([int(r[1]) for r in rows])
    cart = np.array([[float(x) for x in r[2:5]] for r in rows])
    order = np.argsort(ltype, kind="stable")
    ltype, cart = ltype[order], cart[order]
    frac = np.mod(cart @ np.linalg.inv(lat), 1.0)
    m = int(model.maxNeighborNum)
    ntypes = int(model.ntypes)
    types = (ltype - 1).astype(np.int32)
    ln, idr = neigh.find_neighbore(types, frac, lat, ntypes, m, float(model.Rmax),
                                   [float(model.Rmax)] * ntypes)
    at = torch.tensor(list(model.atom_type), dtype=torch.int32)
    Etot, Ei, F, _, V = model(torch.tensor(ln), torch.tensor(types), at, torch.tensor(idr), 0)
    sd = {k: v.numpy() for k, v in model.state_dict().items()}
    np.savez_compressed(
        os.path.join(HERE, "hfo2_jit.npz"), name="hfo2_jit", dtype="float64",
        lattice=lat[None], frac=frac[None], types=types, atom_type=np.array(list(model.atom_type)),
        m=m, Rmax=float(model.Rmax), Rmin=float(model.Rmin),
        davg=model.davg.numpy(), dstd=model.dstd.numpy(),
        list_sha=sha(ln), imagedr_sha=sha(idr), nneigh=(ln > 0).sum(-1).astype(np.int32),
        Etot=Etot.detach().numpy(), Ei=Ei.detach().numpy(), Force=F.detach().numpy(),
        Virial=V.detach().numpy(), **{"w:" + k: v for k, v in sd.items()})
    print("hfo2_jit E", Etot.item(), "max|F|", F.abs().max().item())


def main():
    cu = structures.fcc(3.615, (3, 3, 3), 0.05, seed=11)
    cfg1 = P.DPConfig(atom_type=[29], maxNeighborNum=100)
    seeded_case("cu108_f64", cu, cfg1, seed_w=101, dtype="float64", keep_dE=True)
    seeded_case("cu108_f32", cu, cfg1, seed_w=101, dtype="float32")
    cu2 = structures.fcc(3.615, (3, 3, 3), 0.05, seed=12)
    seeded_case("cu108x2_f64", cu, cfg1, seed_w=102, dtype="float64", batch_structs=[cu2])
    lisi = structures.random_packed(600, 0.05, [3, 14], [0.5, 0.5], seed=21)
    cfg2 = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150)
    seeded_case("lisi600_f64", lisi, cfg2, seed_w=201, dtype="float64")
    hfo = structures.random_packed(48, 0.07, [72, 8], [1 / 3, 2 / 3], seed=31, strain=0.03)
    cfg3 = P.DPConfig(atom_type=[72, 8], maxNeighborNum=100)
    seeded_case("hfo48_f64", hfo, cfg3, seed_w=301, dtype="float64")
    jit_case()


if __name__ == "__main__":
    main()
