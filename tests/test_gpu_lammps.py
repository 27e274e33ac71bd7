"""LAMMPS pair path on the GPU: the slot conversion (matpl_lammps_dp_neighbors) bit-exact
against the oracle restatement of generate_neighdata, and the pair driver
(matpl_lammps_dp_compute) against MatPL's shipped TorchScript model on a LAMMPS-like layout,
against the oracle pair step, and (ghost forces folded) against the periodic path."""
import platform

import numpy as np
import pytest
import torch

from matpl_gb300 import _lib, dp, ops, params as P, structures
from matpl_gb300.lammps import (PairMATPL, firstneigh_of, fold_ghosts, lammps_dp_neighbors,
                                lammps_system)
from oracle import lammps as OL, neigh

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def lmp(golden_case):
    from tests.conftest import load_golden
    g = load_golden("lmp_hfo2_jit")
    base = golden_case(str(g["weights_from"]))
    cfg = P.DPConfig(atom_type=[int(a) for a in g["atom_type"]], maxNeighborNum=int(g["m"]),
                     Rmax=float(g["Rmax"]), Rmin=float(g["Rmin"]))
    s = {"x": g["x"], "type": g["type"], "nlocal": int(g["nlocal"]), "nghost": int(g["nghost"]),
         "owner": g["owner"], "ilist": np.arange(int(g["nlocal"]), dtype=np.int32),
         "jstart": g["jstart"], "jflat": g["jflat"]}
    s["numneigh"] = np.diff(g["jstart"]).astype(np.int32)
    return g, cfg, base, s


def gpu_slots(s, t2m, nt, m, rc, dtype):
    t = lambda a, d: torch.tensor(np.ascontiguousarray(a), dtype=d, device=DEV)
    r = lammps_dp_neighbors(t(s["ilist"], torch.int32), t(s["jstart"], torch.int64),
                            t(s["jflat"], torch.int32), t(s["x"], torch.float64),
                            t(s["type"], torch.int32), t(t2m, torch.int32), nt, m, rc, dtype)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in r.items()}


def mixed_system(natoms, seed, cut=7.0):
    st = structures.random_packed(natoms, 0.05, [3, 14], [0.5, 0.5], seed=seed)
    return st, lammps_system(st.lattice, st.cart, st.types + 1, cut, seed=seed)


def stats(cfg, st):
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, cfg.ntypes, cfg.maxNeighborNum,
                                   cfg.Rmax, [cfg.Rmax] * cfg.ntypes)
    davg, dstd = P.calc_stat(cfg, ln, idr, st.types)
    return torch.as_tensor(davg), torch.as_tensor(dstd)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_slots_bit_exact_vs_oracle(lmp, dtype):
    g, cfg, base, s = lmp
    t2m = [cfg.atom_type.index(int(z)) for z in g["pair_coeff"]]
    ln, dr, tm, mn, ov = OL.neighdata(s["ilist"], s["jstart"], s["jflat"], s["x"], s["type"], t2m,
                                      cfg.ntypes, cfg.maxNeighborNum, cfg.Rmax)
    r = gpu_slots(s, t2m, cfg.ntypes, cfg.maxNeighborNum, cfg.Rmax, dtype)
    assert int(r["err"][0]) == 0
    assert np.array_equal(r["list_neigh"], ln)
    want = dr if dtype == torch.float64 else dr.astype(np.float32)
    assert np.array_equal(r["ImageDR"], want)
    assert np.array_equal(r["Imagetype_map"], tm)
    assert r["min_rsq"][0] == mn


@pytest.mark.parametrize("natoms,m", [(600, 150), (4000, 150)])
def test_slots_two_types_random_lists(natoms, m):
    st, s = mixed_system(natoms, seed=natoms)
    for t2m in ([0, 1], [1, 0]):
        ln, dr, tm, mn, ov = OL.neighdata(s["ilist"], s["jstart"], s["jflat"], s["x"], s["type"],
                                          t2m, 2, m, 6.0)
        assert not ov
        r = gpu_slots(s, t2m, 2, m, 6.0, torch.float64)
        assert int(r["err"][0]) == 0
        assert np.array_equal(r["list_neigh"], ln) and np.array_equal(r["ImageDR"], dr)
        assert np.array_equal(r["Imagetype_map"], tm) and r["min_rsq"][0] == mn


def test_slots_overflow_empty_and_bad_index():
    st, s = mixed_system(600, seed=5)
    r = gpu_slots(s, [0, 1], 2, 10, 6.0, torch.float64)
    assert int(r["err"][0]) == _lib.KERR_NEIGHBOR_OVERFLOW
    # empty lists: all slots zero, no pair
    e = dict(s, jstart=np.zeros(s["nlocal"] + 1, np.int64), jflat=np.zeros(0, np.int32))
    r = gpu_slots(e, [0, 1], 2, 150, 6.0, torch.float64)
    assert int(r["err"][0]) == 0 and r["list_neigh"].sum() == 0 and r["ImageDR"].sum() == 0
    assert r["min_rsq"][0] == 1e300
    # a list entry outside the atoms is flagged and skipped
    b = dict(s, jflat=s["jflat"].copy())
    b["jflat"][3] = s["x"].shape[0] + 4
    r = gpu_slots(b, [0, 1], 2, 150, 6.0, torch.float64)
    assert int(r["err"][0]) == _lib.KERR_BAD_COUNT


ACCESS = ["staged", "direct"]


def pair_of(cfg, params, davg, dstd, precision, pair_coeff, grouped=True, access="staged"):
    model = dp.DP(cfg, params, davg, dstd, precision=precision, device=DEV)
    return PairMATPL(model, pair_coeff, eatom_grouped=grouped, host_access=access)


def run_pair(pair, s, eflag_atom=True):
    return pair.compute(s["x"], s["type"], s["nlocal"], s["nghost"], s["ilist"], s["numneigh"],
                        firstneigh_of(s), eflag_atom=eflag_atom)


@pytest.mark.parametrize("access", ACCESS)
def test_pair_matches_torchscript_model(lmp, access):
    """pair_coeff * * 72 8 on the demo HfO2 cell: forces on local and ghost rows, energy,
    Voigt virial and type-grouped per-atom energies = jit_dp.pt's (FP64); both ways of reaching
    LAMMPS' host arrays."""
    g, cfg, base, s = lmp
    pair = pair_of(cfg, base.params, base.davg, base.dstd, "float64",
                   [int(z) for z in g["pair_coeff"]], access=access)
    assert pair.host_access == access
    r = run_pair(pair, s)
    fs = np.abs(g["Force"]).max()
    np.testing.assert_allclose(r["f"], g["Force"][0], rtol=0, atol=1e-10 * fs)
    np.testing.assert_allclose(r["eng"], g["Etot"].item(), rtol=1e-12)
    np.testing.assert_allclose(r["eatom"], g["Ei"][0], rtol=0, atol=1e-10)
    V = g["Virial"][0]
    np.testing.assert_allclose(r["virial"], V[[0, 4, 8, 1, 2, 5]], rtol=0,
                               atol=1e-10 * np.abs(V).max())
    assert r["min_rsq"] == float(g["min_rsq"])
    # a second call reuses the handle's buffers and gives the same answer (up to the order of
    # the force scatter's atomic adds)
    r2 = run_pair(pair, s)
    np.testing.assert_allclose(r2["f"], r["f"], rtol=0, atol=1e-12 * fs)
    np.testing.assert_allclose(r2["eng"], r["eng"], rtol=1e-13)
    pair.close()


def test_auto_host_access_is_direct_on_grace():
    """On a GPU that reads pageable host memory through the host's page tables the automatic
    choice is the in-place form."""
    cfg = P.DPConfig(atom_type=[29], maxNeighborNum=100)
    st = structures.fcc(3.615, (3, 3, 3), 0.05, seed=1)
    davg, dstd = stats(cfg, st)
    pair = pair_of(cfg, P.init_params(cfg, 1), davg, dstd, "float64", [29], access="auto")
    assert pair.host_access in ("direct", "staged")
    if platform.machine() == "aarch64":
        assert pair.host_access == "direct"
    pair.close()


@pytest.mark.parametrize("precision,tol", [("float64", 1e-10), ("float32", 2e-5),
                                           ("mixed", 2e-5)])
@pytest.mark.parametrize("access", ACCESS)
def test_pair_matches_oracle_two_types(precision, tol, access):
    st, s = mixed_system(600, seed=21)
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150)
    params = P.init_params(cfg, 201)
    davg, dstd = stats(cfg, st)
    s["numneigh"] = np.diff(s["jstart"]).astype(np.int32)
    for pc in ([3, 14], [14, 3]):
        t2m = [cfg.atom_type.index(z) for z in pc]
        # LAMMPS type k is element pc[k-1]; keep the structure's elements
        lt = np.array([pc.index(cfg.atom_type[t]) + 1 for t in st.types], dtype=np.int32)
        sk = dict(s, type=lt[s["owner"]])
        ref = OL.pair_compute(cfg, params, davg, dstd, t2m, sk["nlocal"], sk["nghost"],
                              sk["ilist"], sk["jstart"], sk["jflat"], sk["x"], sk["type"])
        for grouped in (True, False):
            pair = pair_of(cfg, params, davg, dstd, precision, pc, grouped, access)
            r = run_pair(pair, sk)
            fs = np.abs(ref["f"]).max()
            np.testing.assert_allclose(r["f"], ref["f"], rtol=0, atol=tol * fs * 10)
            np.testing.assert_allclose(r["eng"], ref["eng"], rtol=0,
                                       atol=tol * np.abs(ref["eatom"]).sum())
            np.testing.assert_allclose(r["virial"], ref["virial"], rtol=0,
                                       atol=tol * np.abs(ref["virial"]).max() * 10)
            ea = ref["eatom"] if grouped else ref["eatom_atom"]
            np.testing.assert_allclose(r["eatom"], ea, rtol=0, atol=tol * np.abs(ea).max() * 10)
            pair.close()


@pytest.mark.parametrize("access", ACCESS)
def test_pair_ghosts_fold_to_periodic_path(access):
    """Cu, 4000 atoms: ghost forces folded onto their owners = the periodic matpl path."""
    st = structures.fcc(3.615, (10, 10, 10), 0.05, seed=4)
    cfg = P.DPConfig(atom_type=[29], maxNeighborNum=100)
    params = P.init_params(cfg, 101)
    davg, dstd = stats(cfg, st)
    s = lammps_system(st.lattice, st.cart, st.types + 1, 7.0, seed=4)
    model = dp.DP(cfg, params, davg, dstd, precision="float64", device=DEV)
    pair = PairMATPL(model, [29], host_access=access)
    r = run_pair(pair, s)
    n = s["nlocal"]
    lat = torch.tensor(st.lattice[None], device=DEV)
    frac = torch.tensor(np.mod(s["x"][:n] @ np.linalg.inv(st.lattice), 1.0)[None], device=DEV)
    ln, idr = ops.find_neighbore(torch.zeros(n, dtype=torch.int32), frac, lat, 1, 100, 6.0, 6.0)
    tmap = torch.zeros(n, dtype=torch.int32, device=DEV)
    out = model.evaluate(ln, tmap, [0], idr, 0)
    Ff = fold_ghosts(r["f"], s["owner"], n)
    F = out["Force"][0].cpu().numpy()
    np.testing.assert_allclose(Ff, F, rtol=0, atol=1e-10 * np.abs(F).max())
    np.testing.assert_allclose(r["eng"], out["Etot"].item(), rtol=1e-12)
    V = out["Virial"][0].cpu().numpy()
    np.testing.assert_allclose(r["virial"], V[[0, 4, 8, 3, 6, 7]], rtol=0,
                               atol=1e-10 * np.abs(V).max())
    pair.close()


@pytest.mark.parametrize("access", ACCESS)
def test_pair_too_close_and_sizes_change(access):
    st, s = mixed_system(600, seed=9)
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150)
    params = P.init_params(cfg, 7)
    davg, dstd = stats(cfg, st)
    s["numneigh"] = np.diff(s["jstart"]).astype(np.int32)
    pair = pair_of(cfg, params, davg, dstd, "float64", [3, 14], access=access)
    r_big = run_pair(pair, s)
    st2, s2 = mixed_system(100, seed=10)
    s2["numneigh"] = np.diff(s2["jstart"]).astype(np.int32)
    run_pair(pair, s2)
    r_again = run_pair(pair, s)
    np.testing.assert_allclose(r_again["f"], r_big["f"], rtol=0,
                               atol=1e-12 * np.abs(r_big["f"]).max())
    # move atom 1's first neighbor onto it: the reference stops the run (rsq < 0.61)
    c = dict(s, x=s["x"].copy())
    j = int(s["jflat"][s["jstart"][1]])
    c["x"][j] = c["x"][1] + np.array([0.3, 0.0, 0.0])
    with pytest.raises(_lib.MatplError, match="too close"):
        run_pair(pair, c)
    # inum == 0 writes nothing
    f0 = np.full((3, 3), 7.0)
    pair.compute(np.zeros((3, 3)), np.ones(3, np.int32), 0, 3, np.zeros(0, np.int32),
                 np.zeros(0, np.int32), np.zeros(0, np.uint64), f_out=f0)
    assert (f0 == 7.0).all()
    pair.close()


@pytest.mark.parametrize("access", ACCESS)
def test_model_deviation_shares_one_conversion(access):
    """Three models on one slot conversion (compute_models) = each model's own pair step; the
    deviation of identical models is zero; models must share ntypes, m and Rmax."""
    from matpl_gb300.lammps import compute_models, model_deviation
    st, s = mixed_system(600, seed=31)
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150)
    davg, dstd = stats(cfg, st)
    s["numneigh"] = np.diff(s["jstart"]).astype(np.int32)
    models = [dp.DP(cfg, P.init_params(cfg, 300 + k), davg, dstd, precision="float64",
                    device=DEV) for k in range(3)]
    pair = PairMATPL(models[0], [3, 14], host_access=access)
    for mdl in models[1:]:
        pair.add_model(mdl)
    r = compute_models(pair, s["x"], s["type"], s["nlocal"], s["nghost"], s["ilist"],
                       s["numneigh"], firstneigh_of(s))
    assert r["f"].shape == (3, s["nlocal"] + s["nghost"], 3)
    for k, mdl in enumerate(models):
        one = PairMATPL(mdl, [3, 14], host_access=access)
        o = run_pair(one, s)
        np.testing.assert_allclose(r["f"][k], o["f"], rtol=0, atol=1e-12 * np.abs(o["f"]).max())
        np.testing.assert_allclose(r["eng"][k], o["eng"], rtol=1e-13)
        np.testing.assert_allclose(r["virial"][k], o["virial"], rtol=0,
                                   atol=1e-12 * np.abs(o["virial"]).max())
        np.testing.assert_allclose(r["eatom"][k], o["eatom"], rtol=0, atol=1e-13)
        one.close()
    n = s["nlocal"]
    f_fold = np.stack([fold_ghosts(r["f"][k], s["owner"], n) for k in range(3)])
    dev = model_deviation(f_fold, r["eatom"])
    assert dev[1] >= dev[0] / np.sqrt(3) and dev[1] >= dev[2] >= 0 and dev[4] >= dev[5] >= 0
    same = model_deviation(np.stack([f_fold[0]] * 3), np.stack([r["eatom"][0]] * 3))
    assert max(same) < 1e-12
    other = P.DPConfig(atom_type=[3, 14], maxNeighborNum=120)
    bad = dp.DP(other, P.init_params(other, 1), davg[:, :120 * 2 * 4], dstd[:, :120 * 2 * 4],
                precision="float64", device=DEV)
    with pytest.raises(_lib.MatplError, match="share ntypes"):
        pair.add_model(bad)
    pair.close()


def test_pair_with_compressed_model_folds_to_periodic_path():
    """A compressed model (order-5 table) in the pair style: ghost forces folded onto their
    owners, energy and virial = the same compressed model on the periodic cell (FP64)."""
    from matpl_gb300 import compress as C
    st = structures.fcc(3.615, (8, 8, 8), 0.05, seed=5)
    cfg = P.DPConfig(atom_type=[29], maxNeighborNum=100)
    params = P.init_params(cfg, 103)
    davg, dstd = stats(cfg, st)
    comp = C.build_table(cfg, params, davg.numpy(), dstd.numpy(), 2.5, 0.01, 5, device=DEV)
    model = C.fused_model(cfg, params, davg, dstd, comp, "float64", DEV)
    s = lammps_system(st.lattice, st.cart, st.types + 1, 7.0, seed=5)
    pair = PairMATPL(model, [29], host_access="staged")
    r = run_pair(pair, s)
    n = s["nlocal"]
    lat = torch.tensor(st.lattice[None], device=DEV)
    frac = torch.tensor(np.mod(s["x"][:n] @ np.linalg.inv(st.lattice), 1.0)[None], device=DEV)
    ln, idr = ops.find_neighbore(torch.zeros(n, dtype=torch.int32), frac, lat, 1, 100, 6.0, 6.0)
    out = model.evaluate(ln, torch.zeros(n, dtype=torch.int32, device=DEV), [0], idr, 0)
    F = out["Force"][0].cpu().numpy()
    np.testing.assert_allclose(fold_ghosts(r["f"], s["owner"], n), F, rtol=0,
                               atol=1e-10 * np.abs(F).max())
    np.testing.assert_allclose(r["eng"], out["Etot"].item(), rtol=1e-12)
    V = out["Virial"][0].cpu().numpy()
    np.testing.assert_allclose(r["virial"], V[[0, 4, 8, 3, 6, 7]], rtol=0,
                               atol=1e-10 * np.abs(V).max())
    assert int(model.err.item()) == 0
    pair.close()
