"""Generate the golden fixture of the LAMMPS DP pair step from MatPL's shipped TorchScript model.

Runs only where the MatPL source tree is mounted (path in MATPL_REF, default: a
``reference`` directory beside the repository root);
the committed ``lmp_hfo2_jit.npz`` is what the tests read.  It

1. reads the demo structure ``src/lmps/lammps-libtorch/dp_lmps_demo/lmp.config`` (96 atoms of
   HfO2, triclinic) and the demo's settings (``in.lammps``: ``pair_coeff * * 72 8``,
   ``neighbor 1.0 bin``),
2. builds LAMMPS-like local + ghost atoms and a full neighbor list in random order within
   Rmax + 1.0 (``matpl_gb300.lammps.lammps_system``),
3. converts the list into DP slots with the oracle restatement of
   ``PairMATPL::generate_neighdata`` (``oracle/lammps_neigh.c``),
4. runs the TorchScript model ``jit_dp.pt`` exactly as ``pair_matpl.cpp:932`` does
   (``forward(list_neigh, imagetype_map, atom_type, dR, nghost)``),
5. stores the system (positions, types, list), the slot checksums and the model's outputs.
   The weights, davg and dstd are those of ``hfo2_jit.npz`` (the same model; checked here).

Usage:  python tests/golden/make_lammps_golden.py
"""
import hashlib
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from matpl_gb300.lammps import lammps_system  # noqa: E402
from oracle import lammps as OL  # noqa: E402

from oracle.refpath import reference_root  # noqa: E402

REF = reference_root()
SKIN = 1.0
PAIR_COEFF = [72, 8]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def read_config(path):
    lines = open(path).read().splitlines()
    nat = int([l for l in lines if l.strip().endswith("atoms")][0].split()[0])
    lo_hi = [list(map(float, [l for l in lines if l.strip().endswith(f"{a}lo {a}hi")][0]
                           .split()[:2])) for a in "xyz"]
    xy, xz, yz = map(float, [l for l in lines if l.strip().endswith("xy xz yz")][0].split()[:3])
    lat = np.array([[lo_hi[0][1] - lo_hi[0][0], 0, 0], [xy, lo_hi[1][1] - lo_hi[1][0], 0],
                    [xz, yz, lo_hi[2][1] - lo_hi[2][0]]])
    start = [i for i, l in enumerate(lines) if l.strip().startswith("Atoms")][0] + 2
    rows = [l.split() for l in lines[start:start + nat]]
    ltype = np.array([int(r[1]) for r in rows], dtype=np.int32)
    cart = np.array([[float(v) for v in r[2:5]] for r in rows])
    return lat, cart, ltype


def main():
    demo = os.path.join(REF, "src/lmps/lammps-libtorch/dp_lmps_demo")
    model = torch.jit.load(os.path.join(demo, "jit_dp.pt"))
    lat, cart, ltype = read_config(os.path.join(demo, "lmp.config"))
    rmax = float(model.Rmax)
    m = int(model.maxNeighborNum)
    at = [int(a) for a in model.atom_type]
    t2m = [at.index(z) for z in PAIR_COEFF]
    sysd = lammps_system(lat, cart, ltype, rmax + SKIN, seed=7)
    ln, dr, tm, mn, ov = OL.neighdata(sysd["ilist"], sysd["jstart"], sysd["jflat"], sysd["x"],
                                      sysd["type"], t2m, len(at), m, rmax)
    assert not ov
    nghost = sysd["nghost"]
    Etot, Ei, F, _, V = model(torch.tensor(ln), torch.tensor(tm),
                              torch.tensor(PAIR_COEFF, dtype=torch.int32), torch.tensor(dr),
                              nghost)
    base = dict(np.load(os.path.join(HERE, "hfo2_jit.npz")))
    for k, v in model.state_dict().items():
        assert np.array_equal(base["w:" + k], v.numpy()), k
    assert np.array_equal(base["davg"], model.davg.numpy())
    assert np.array_equal(base["dstd"], model.dstd.numpy())
    np.savez_compressed(
        os.path.join(HERE, "lmp_hfo2_jit.npz"), name="lmp_hfo2_jit", lattice=lat,
        x=sysd["x"], type=sysd["type"], owner=sysd["owner"].astype(np.int32),
        nlocal=sysd["nlocal"], nghost=nghost, jstart=sysd["jstart"], jflat=sysd["jflat"],
        pair_coeff=np.array(PAIR_COEFF), skin=SKIN, atom_type=np.array(at), m=m, Rmax=rmax,
        Rmin=float(model.Rmin), weights_from="hfo2_jit", list_sha=sha(ln), imagedr_sha=sha(dr),
        type_map=tm, min_rsq=mn,
        Etot=Etot.detach().numpy(), Ei=Ei.detach().numpy(), Force=F.detach().numpy(),
        Virial=V.detach().numpy())
    print("lmp_hfo2_jit nlocal", sysd["nlocal"], "nghost", nghost, "list entries",
          sysd["jflat"].size, "E", Etot.item(), "max|F|", F.abs().max().item(), "min_rsq", mn)


if __name__ == "__main__":
    main()
