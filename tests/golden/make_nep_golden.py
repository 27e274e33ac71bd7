"""Generate the NEP golden fixtures by running MatPL's own NEP implementation.

Runs only where the MatPL source tree is mounted (path in MATPL_REF, default: a
``reference`` directory beside the repository root);
the committed ``nep_*.npz`` files are what the tests read.  For each case it

1. builds seeded synthetic frames (``matpl_gb300.structures``) and expands their boxes with
   ``matpl_gb300.nep.expand_box`` (the restatement of ``UniDataset.expand_box``; the fixture keeps
   the box arrays, so the reference's neighbor operator below sees exactly these inputs),
2. compiles the reference's CPU operator library from its own sources (``oracle/ref_build.py``)
   and runs ``CalcOps_cpu.calculate_maxneigh`` and ``calculate_neighbor`` (with_rij = True),
3. builds the reference ``src.model.nep_net.NEP`` (its CPU branch) with seeded parameters, sets
   q_scaler with the reference's own ``update_scaler_values`` on the case's descriptors, and
   evaluates ``forward`` in FP64,
4. stores the inputs, the seeds, checksums of the neighbor lists, the descriptors and E/F/V.

Usage:  python tests/golden/make_nep_golden.py [case names]   (default: every case)
"""
import hashlib
import os
import sys
import types as _types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from matpl_gb300 import nep as NP, structures  # noqa: E402
from oracle import ref_build  # noqa: E402

from oracle.refpath import reference_root  # noqa: E402

REF = reference_root()


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def reference_nep_class():
    """Import src.model.nep_net with torch.ops.load_library pointed at the library built from
    the reference's sources (nep_net.py:17-24 loads it from a fixed path in the source tree)."""
    ops = ref_build.load()
    real = torch.ops.load_library
    torch.ops.load_library = lambda path: None
    try:
        sys.path.insert(0, REF)
        sys.path.insert(0, os.path.join(REF, "src"))
        from src.model import nep_net
    finally:
        torch.ops.load_library = real
    return nep_net.NEP, ops


def fake_input_param(cfg: NP.NepConfig):
    nep_param = _types.SimpleNamespace(
        zbl=cfg.zbl, c2_param=None, c3_param=None, q_scaler=None, model_wb=None,
        bias_lastlayer=None, cutoff=list(cfg.cutoff), n_max=list(cfg.n_max),
        basis_size=list(cfg.basis_size), l_max=list(cfg.l_max), neuron=[cfg.neuron, 1],
        train_2b=cfg.train_2b)
    return _types.SimpleNamespace(model_type="NEP", nep_param=nep_param, precision="float64",
                                  atom_type=list(cfg.atom_type), max_neigh_num=100)


def run_case(name, cfg: NP.NepConfig, structs, seed_w, NEP, ops):
    fr = NP.frames_from_structures(structs, cfg.cutoff[0])
    t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt)  # noqa: E731
    num_atom = t(fr.num_atom.reshape(-1, 1), torch.int64)  # collated [B, 1] (nep_data_loader.py:210)
    tmap = t(fr.type_map, torch.int64)
    box, bo = t(fr.box, torch.float64), t(fr.box_orig, torch.float64)
    nc, pos = t(fr.num_cell, torch.int64), t(fr.position, torch.float64)
    cnt_r, cnt_a = ops.calculate_maxneigh(num_atom, box, bo, nc, pos, cfg.cutoff[0],
                                          cfg.cutoff[1], cfg.ntypes, tmap, False)
    max_r, max_a = int(cnt_r.max()) + 3, int(cnt_a.max()) + 3
    ftype = t(np.arange(cfg.ntypes), torch.int64)
    NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = ops.calculate_neighbor(
        num_atom, tmap, ftype, box, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], max_r, max_a, True)

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
    model.set_nep_param_device(q_scaler=np.ones(cfg.feature_nums))

    captured = {}
    real_qn = model.calculate_qn

    def qn(*a, **k):
        out = real_qn(*a, **k)
        captured["feats"] = out.detach().clone()
        return out
    model.calculate_qn = qn

    def forward():
        return model(NN_r.clone(), NL_r.clone(), Ri_r.clone(), NN_a.clone(), NL_a.clone(),
                     Ri_a.clone(), num_atom, tmap)

    forward()
    feats = captured["feats"]
    dt = feats.dtype
    qmax0 = torch.full([cfg.feature_nums], -float("inf"), dtype=dt)
    qmin0 = torch.full([cfg.feature_nums], float("inf"), dtype=dt)
    qmax, qmin = model.update_scaler_values(feats, cfg.two_feat_num,
                                            cfg.na * cfg.l_max[0], cfg.n_max[1], qmax0, qmin0,
                                            *cfg.l_max)
    q_scaler = (1.0 / (qmax - qmin)).detach()
    model.reset_scaler(q_scaler.numpy(), torch.float64, "cpu")
    Etot, Ei, Force, _, Virial = forward()

    rec = dict(
        name=name, seed_w=seed_w, atom_type=np.array(cfg.atom_type), cutoff=np.array(cfg.cutoff),
        n_max=np.array(cfg.n_max), basis_size=np.array(cfg.basis_size),
        l_max=np.array(cfg.l_max), neuron=cfg.neuron, train_2b=cfg.train_2b,
        zbl=np.nan if cfg.zbl is None else float(cfg.zbl),
        position=fr.position, type_map=fr.type_map, num_atom=fr.num_atom, box=fr.box,
        box_orig=fr.box_orig, num_cell=fr.num_cell, lattice=np.stack([s.lattice for s in structs]),
        max_r=max_r, max_a=max_a, cnt_r=cnt_r.numpy(), cnt_a=cnt_a.numpy(),
        NN_r=NN_r.numpy(), NN_a=NN_a.numpy(), NL_r=NL_r.numpy(),
        NL_a=NL_a.numpy(), sha_Ri_r=sha(Ri_r.numpy()), sha_Ri_a=sha(Ri_a.numpy()),
        sha_NL_r=sha(NL_r.numpy()), sha_NL_a=sha(NL_a.numpy()),
        q_scaler=q_scaler.numpy(), feats=feats.numpy(), Etot=Etot.detach().numpy(),
        Ei=Ei.detach().numpy(), Force=Force.detach().numpy(), Virial=Virial.detach().numpy())
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "atoms", fr.natoms, "frames", fr.nframes, "num_cell", fr.num_cell.tolist(),
          "max_r", max_r, "max_a", max_a, "Etot", Etot.detach().numpy().ravel())


def main(which=None):
    NEP, ops = reference_nep_class()
    want = (lambda n: which is None or n in which)  # noqa: E731
    cfg4 = NP.NepConfig(atom_type=[3, 14, 8, 72])
    if want("nep_q4_240"):
        st = structures.random_packed(240, 0.06, [3, 14, 8, 72], [0.25] * 4, seed=41)
        run_case("nep_q4_240", cfg4, [st], seed_w=401, NEP=NEP, ops=ops)
    # two triclinic frames, small enough that the box is replicated (num_cell > 1)
    if want("nep_q4_tri2"):
        a = structures.random_packed(40, 0.06, [3, 14, 8, 72], [0.25] * 4, seed=42, strain=0.04)
        b = structures.random_packed(64, 0.06, [3, 14, 8, 72], [0.25] * 4, seed=43, strain=0.04)
        run_case("nep_q4_tri2", cfg4, [a, b], seed_w=402, NEP=NEP, ops=ops)
    # 3-body only (no 4-body / 5-body), two elements, a wider hidden layer
    if want("nep_hfo_l4"):
        cfg_b = NP.NepConfig(atom_type=[8, 72], cutoff=(5.0, 3.5), n_max=(3, 5),
                             basis_size=(6, 7), l_max=(4, 0, 0), neuron=40)
        c = structures.random_packed(150, 0.07, [8, 72], [2 / 3, 1 / 3], seed=44, strain=0.02)
        run_case("nep_hfo_l4", cfg_b, [c], seed_w=403, NEP=NEP, ops=ops)
    # the ZBL term (outer cutoff 2.2 A, inner 1.1 A): atoms packed down to 0.9 A (first frame)
    # and 1.3 A (second) so that pairs fall in both the inner and the switching region
    if want("nep_zbl"):
        cfg_z = NP.NepConfig(atom_type=[3, 14, 8, 72], zbl=2.2)
        a = structures.random_packed(96, 0.07, [3, 14, 8, 72], [0.25] * 4, seed=45,
                                     min_dist=0.9)
        b = structures.random_packed(80, 0.07, [3, 14, 8, 72], [0.25] * 4, seed=46,
                                     min_dist=1.3, strain=0.03)
        run_case("nep_zbl", cfg_z, [a, b], seed_w=404, NEP=NEP, ops=ops)


if __name__ == "__main__":
    main(set(sys.argv[1:]) or None)
