"""CPU checks of the LAMMPS pair path: the oracle restatement of generate_neighdata and the
reference's DP pair step against MatPL's shipped TorchScript model run on a LAMMPS-like layout
(local + ghost atoms, full list in random order), the ghost-atom physics against the periodic
path, and the host-side argument checks of the C ABI."""
import ctypes
import hashlib

import numpy as np
import pytest
import torch

from matpl_gb300 import _lib, params as P, structures
from matpl_gb300.lammps import fold_ghosts, lammps_system
from oracle import dp_oracle, lammps as OL, neigh


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def lmp(golden_case):
    from tests.conftest import load_golden
    g = load_golden("lmp_hfo2_jit")
    base = golden_case(str(g["weights_from"]))
    cfg = P.DPConfig(atom_type=[int(a) for a in g["atom_type"]], maxNeighborNum=int(g["m"]),
                     Rmax=float(g["Rmax"]), Rmin=float(g["Rmin"]))
    t2m = [cfg.atom_type.index(int(z)) for z in g["pair_coeff"]]
    return g, cfg, base.params, base.davg, base.dstd, t2m


def test_oracle_pair_step_matches_torchscript_model(lmp):
    """generate_neighdata restatement + DP oracle with ghost rows = jit_dp.pt's outputs."""
    g, cfg, params, davg, dstd, t2m = lmp
    n, ng = int(g["nlocal"]), int(g["nghost"])
    r = OL.pair_compute(cfg, params, davg, dstd, t2m, n, ng, np.arange(n), g["jstart"],
                        g["jflat"], g["x"], g["type"])
    assert _sha(r["list_neigh"]) == str(g["list_sha"])
    assert _sha(r["image_dr"]) == str(g["imagedr_sha"])
    assert np.array_equal(r["type_map"], g["type_map"])
    assert r["min_rsq"] == float(g["min_rsq"])
    assert r["f"].shape == (n + ng, 3)
    np.testing.assert_allclose(r["eng"], g["Etot"].item(), rtol=1e-12)
    np.testing.assert_allclose(r["eatom"], g["Ei"][0], rtol=0, atol=1e-11)
    fs = np.abs(g["Force"]).max()
    np.testing.assert_allclose(r["f"], g["Force"][0], rtol=0, atol=1e-11 * fs)
    V = g["Virial"][0]
    np.testing.assert_allclose(r["virial"], V[[0, 4, 8, 1, 2, 5]], rtol=0,
                               atol=1e-11 * np.abs(V).max())


def test_ghost_layout_equals_periodic_cell(lmp):
    """Ghost forces folded onto their owners (LAMMPS reverse communication) give the forces of
    the periodic cell; energy and virial are those of the periodic cell."""
    g, cfg, params, davg, dstd, t2m = lmp
    n = int(g["nlocal"])
    lat = g["lattice"]
    types = np.array([t2m[t - 1] for t in g["type"][:n]], dtype=np.int32)
    frac = np.mod(g["x"][:n] @ np.linalg.inv(lat), 1.0)
    ln, idr = neigh.find_neighbore(types, frac, lat, cfg.ntypes, cfg.maxNeighborNum, cfg.Rmax,
                                   [cfg.Rmax] * cfg.ntypes)
    out = dp_oracle.dp_eval(cfg, params, davg, dstd, torch.tensor(ln), torch.tensor(types),
                            torch.tensor([cfg.atom_type[t] for t in t2m]), torch.tensor(idr), 0)
    np.testing.assert_allclose(out["Etot"].item(), g["Etot"].item(), rtol=1e-12)
    Ff = fold_ghosts(g["Force"][0], g["owner"], n)
    np.testing.assert_allclose(Ff, out["Force"][0].detach().numpy(), rtol=0, atol=1e-10)
    np.testing.assert_allclose(g["Virial"][0], out["Virial"][0].detach().numpy(), rtol=0,
                               atol=1e-9)


def test_oracle_overflow_and_empty_rows():
    st = structures.fcc(3.615, (3, 3, 3), 0.05, seed=3)
    s = lammps_system(st.lattice, st.cart, st.types + 1, 7.0, seed=1)
    n = s["nlocal"]
    ln, dr, tm, mn, ov = OL.neighdata(s["ilist"], s["jstart"], s["jflat"], s["x"], s["type"],
                                      [0], 1, 100, 6.0)
    assert not ov and (ln > 0).sum(-1).max() <= 100 and mn < 1000
    # order inside a type block is the list order
    row = s["jflat"][s["jstart"][5]:s["jstart"][6]]
    d = s["x"][row] - s["x"][5]
    kept = row[(d * d).sum(1) <= 36.0]
    assert np.array_equal(ln[0, 5, :kept.size], kept + 1)
    _, _, _, _, ov = OL.neighdata(s["ilist"], s["jstart"], s["jflat"], s["x"], s["type"], [0], 1,
                                  20, 6.0)
    assert ov
    # atoms with empty lists and an empty list array
    js = np.zeros(n + 1, dtype=np.int64)
    ln, dr, tm, mn, ov = OL.neighdata(s["ilist"], js, np.zeros(0, np.int32), s["x"], s["type"],
                                      [0], 1, 100, 6.0)
    assert not ov and ln.sum() == 0 and dr.sum() == 0 and mn == 1000


def test_lammps_system_ghost_rule():
    st = structures.fcc(3.615, (2, 2, 2), 0.0, seed=0)
    s = lammps_system(st.lattice, st.cart, st.types + 1, 5.0, seed=0)
    n = s["nlocal"]
    assert s["nghost"] > 0 and np.array_equal(s["owner"][:n], np.arange(n))
    # every ghost images its owner by a lattice vector
    shift = (s["x"][n:] - s["x"][s["owner"][n:]]) @ np.linalg.inv(st.lattice)
    assert np.allclose(shift, np.round(shift), atol=1e-9)
    # full list = every atom (not i) within the cutoff
    for i in (0, 7, n - 1):
        row = s["jflat"][s["jstart"][i]:s["jstart"][i + 1]]
        r = np.linalg.norm(s["x"] - s["x"][i], axis=1)
        want = np.nonzero(r <= 5.0)[0]
        assert sorted(row.tolist()) == sorted(w for w in want.tolist() if w != i)


def test_capi_lammps_argument_checks():
    lib = _lib.load()
    m = _lib.MatplDpModel()
    m.ntypes, m.m = 2, 100
    h = ctypes.c_void_p()
    t2m = (ctypes.c_int * 2)(1, 1)
    # no parameter pointers
    t2m_p = ctypes.cast(t2m, ctypes.c_void_p)
    assert lib.matpl_lammps_dp_create(1, ctypes.byref(m), 2, t2m_p, 1, 0, ctypes.byref(h)) == 1
    m.params = m.davg = m.dstd = 16
    st = lib.matpl_lammps_dp_create(1, ctypes.byref(m), 2, t2m_p, 1, 0, ctypes.byref(h))
    assert st == 1 and b"same model type" in lib.matpl_last_error()
    assert lib.matpl_lammps_dp_create(9, ctypes.byref(m), 2, t2m_p, 1, 0, ctypes.byref(h)) == 2
    assert lib.matpl_lammps_dp_create(1, ctypes.byref(m), 2, t2m_p, 1, 7, ctypes.byref(h)) == 1
    assert lib.matpl_lammps_dp_host_access(None) == -1
    assert lib.matpl_lammps_dp_compute(None, 1, 0, 1, *([None] * 10)) == 1
    assert lib.matpl_lammps_dp_neighbors(1, 1, *([None] * 6), 1, 2, 100, 6.0, 1,
                                         *([None] * 6)) == 1
