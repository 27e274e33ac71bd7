"""Generate the golden fixture of the data-path statistics from MatPL's own loader code.

Runs only where the MatPL source tree is mounted (path in MATPL_REF, default: a
``reference`` directory beside the repository root);
the committed ``data_stats.npz`` is what the tests read.  It imports
``src/pre_data/dpuni_data_loader.py`` (with stand-ins for the modules it imports but does not
use here: pwdata, yaml, the input-parameter class and the Fortran NeighConst module, which
cannot be compiled without ifort) and runs, on seeded synthetic images of two elements with
uneven sizes and compositions (one image lacks an element):

1. ``calc_stat`` on each image's neighbor lists (the oracle restatement of NeighConst, which
   the tests pin bit for bit) in the layout calculate_davg_dstd hands it,
2. ``UniDataset.set_davg_dstd`` with ``calculate_davg_dstd`` fed by the same lists,
3. ``UniDataset.set_energy_shift`` on the images' synthetic energies,
with Python's ``random`` seeded before 2 and 3 (the loader shuffles with it).

Usage:  python tests/golden/make_data_golden.py
"""
import os
import random
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from matpl_gb300 import params as P, structures  # noqa: E402
from oracle import neigh  # noqa: E402

from oracle.refpath import reference_root  # noqa: E402

REF = reference_root()
ATOM_TYPE = [3, 14]
M, RC, RMIN = 60, 5.0, 0.5
SEED_SHUFFLE = 1234


def images():
    out = []
    specs = [(24, [0.5, 0.5], 1), (24, [0.5, 0.5], 2), (40, [0.25, 0.75], 3), (16, [1.0, 0.0], 4),
             (32, [0.5, 0.5], 5), (24, [0.5, 0.5], 6), (48, [0.75, 0.25], 7), (20, [0.0, 1.0], 8)]
    for n, frac, seed in specs:
        els = [z for z, f in zip(ATOM_TYPE, frac) if f > 0]
        fr = [f for f in frac if f > 0]
        st = structures.random_packed(n, 0.05, els, fr, seed=seed)
        order = np.argsort(st.types, kind="stable")           # atoms grouped by element
        st = structures.Structure(st.lattice, st.frac[order], st.types[order], st.elements)
        out.append(st)
    return out


def load_reference():
    for name in ("pwdata", "pwdata.image", "yaml", "src.user.input_param", "src.lib",
                 "src.lib.NeighConst"):
        mod = types.ModuleType(name)
        sys.modules[name] = mod
    sys.modules["pwdata"].Config = object
    sys.modules["pwdata.image"].Image = object
    sys.modules["src.user.input_param"].InputParam = object
    sys.modules["src.lib.NeighConst"].neighconst = None
    sys.path.insert(0, REF)
    sys.path.insert(0, os.path.join(REF, "src"))
    import torch
    real = torch.ops.load_library
    torch.ops.load_library = lambda path: None      # the module loads the op library it
    try:                                            # does not use here
        from src.pre_data import dpuni_data_loader as dl
    finally:
        torch.ops.load_library = real
    return dl


def main():
    dl = load_reference()
    cfg = P.DPConfig(atom_type=ATOM_TYPE, maxNeighborNum=M, Rmax=RC, Rmin=RMIN)
    config = {"Rc_M": RC, "maxNeighborNum": M,
              "atomType": [{"type": z, "Rc": RC, "Rm": RMIN} for z in ATOM_TYPE]}
    ims = images()
    nt = len(ATOM_TYPE)

    def lists(st):
        tm = np.array([ATOM_TYPE.index(st.elements[t]) for t in st.types], dtype=np.int32)
        ln, idr = neigh.find_neighbore(tm, st.frac, st.lattice, nt, M, RC, [RC] * nt)
        N = st.natoms
        return tm, ln.reshape(1, N, nt, M), idr[..., 1:].reshape(1, N, nt, M, 3)

    def davg_dstd_image(cfg_, lattice, position, _atom_types, input_atom_type, type_maps):
        # calculate_davg_dstd (dpuni_data_loader.py:377-420) with the Fortran search replaced
        st = [s for s in ims if s.frac.shape == position.shape and np.array_equal(s.frac, position)]
        assert len(st) == 1
        _, list_neigh, dR_neigh = lists(st[0])
        types_, idx, nums = np.unique(type_maps, return_index=True, return_counts=True)
        nums = nums[np.argsort(idx)]
        atl = sorted(list(input_atom_type).index(a) for a in list(_atom_types))
        return dl.calc_stat(cfg_, np.copy(dR_neigh[:, :, atl]), np.copy(list_neigh[:, :, atl]),
                            M, position.shape[0], len(atl), nums)

    per_image = []
    for st in ims:
        tm, ln, dr = lists(st)
        _, idx, nums = np.unique(tm, return_index=True, return_counts=True)
        nums = nums[np.argsort(idx)]
        present = sorted(set(tm.tolist()))
        davg, dstd = dl.calc_stat(config, np.copy(dr[:, :, present]), np.copy(ln[:, :, present]),
                                  M, st.natoms, len(present), nums)
        per_image.append((np.array(davg), np.array(dstd)))

    class Img:
        pass
    image_list = []
    rng = np.random.default_rng(9)
    energies = []
    for st in ims:
        im = Img()
        im.atom_types_image = np.asarray(st.elements)[st.types]
        im.lattice = st.lattice
        im.position = st.frac
        e = float(-1.9 * (im.atom_types_image == 3).sum() - 4.7 * (im.atom_types_image == 14).sum()
                  + 0.05 * rng.standard_normal())
        im.Ep = e
        energies.append(e)
        image_list.append(im)
    fake = types.SimpleNamespace(image_list=image_list, atom_types=ATOM_TYPE, config=config)
    dl.calculate_davg_dstd = davg_dstd_image
    random.seed(SEED_SHUFFLE)
    davg, dstd = dl.UniDataset.set_davg_dstd(fake)
    random.seed(SEED_SHUFFLE)
    shift = dl.UniDataset.set_energy_shift(fake)
    rec = {"atom_type": np.array(ATOM_TYPE), "m": M, "Rc": RC, "Rmin": RMIN,
           "seed_shuffle": SEED_SHUFFLE, "energies": np.array(energies),
           "davg": davg, "dstd": dstd, "energy_shift": shift}
    for k, (a, s) in enumerate(per_image):
        rec[f"img{k}_davg"] = a
        rec[f"img{k}_dstd"] = s
    np.savez_compressed(os.path.join(HERE, "data_stats.npz"), **rec)
    print("davg", davg[:, :4], "dstd", dstd[:, :4], "shift", shift)


if __name__ == "__main__":
    main()
