"""NEP on the GPU: neighbor operators bit-exact against the reference fixtures and the oracle,
fused energy / force / virial against the reference fixtures (FP64) and the FP64 oracle."""
import hashlib

import numpy as np
import pytest
import torch

from matpl_gb300 import nep as NP, ops, structures
from oracle import nep_oracle as NO

pytestmark = pytest.mark.gpu
CASES = ["nep_q4_240", "nep_q4_tri2", "nep_hfo_l4"]
DEV = "cuda"


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _t(fr: NP.NepFrames):
    c = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=DEV)  # noqa: E731
    return (c(fr.num_atom.reshape(-1, 1), torch.int64), c(fr.type_map, torch.int64),
            c(fr.box, torch.float64), c(fr.box_orig, torch.float64),
            c(fr.num_cell, torch.int64), c(fr.position, torch.float64))


def gpu_neighbor(fr, cfg, max_r, max_a, with_rij=True):
    na, tm, bx, bo, nc, pos = _t(fr)
    at = torch.arange(cfg.ntypes, device=DEV)
    out = ops.calculate_neighbor(na, tm, at, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1],
                                 max_r, max_a, with_rij)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in out]


def assert_lists_equal(got, exp):
    names = ["NN_r", "NN_a", "NL_r", "NL_a", "Ri_r", "Ri_a"]
    for n, g, e in zip(names, got, exp):
        assert g.shape == e.shape, n
        if not np.array_equal(g.view(np.uint8) if g.dtype == np.float64 else g,
                              e.view(np.uint8) if e.dtype == np.float64 else e):
            bad = np.argwhere(g != e)
            raise AssertionError(f"{n} differs at {bad[:5].tolist()}")


@pytest.mark.parametrize("name", CASES)
def test_neighbor_matches_reference_fixture(nep_case, name):
    c = nep_case(name)
    g = c.g
    NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = gpu_neighbor(c.frames, c.cfg, int(g["max_r"]),
                                                      int(g["max_a"]))
    assert np.array_equal(NN_r, g["NN_r"]) and np.array_equal(NN_a, g["NN_a"])
    assert _sha(NL_r) == str(g["sha_NL_r"]) and _sha(NL_a) == str(g["sha_NL_a"])
    assert _sha(Ri_r) == str(g["sha_Ri_r"]) and _sha(Ri_a) == str(g["sha_Ri_a"])


def _frames(specs, cutoff):
    sts = [structures.random_packed(n, d, [3, 14, 8, 72], [0.25] * 4, seed=s, strain=e)
           for (n, d, s, e) in specs]
    return NP.frames_from_structures(sts, cutoff)


CELL_CASES = {
    "cubic_1500": [(1500, 0.06, 51, 0.0)],
    "tri_2000": [(2000, 0.06, 52, 0.04)],
    "mixed_batch": [(1200, 0.06, 53, 0.02), (60, 0.06, 54, 0.03), (900, 0.07, 55, 0.0)],
}


@pytest.mark.parametrize("case", list(CELL_CASES))
@pytest.mark.parametrize("with_rij", [True, False])
def test_neighbor_cell_list_matches_oracle(case, with_rij):
    cfg = NP.NepConfig(atom_type=[3, 14, 8, 72])
    fr = _frames(CELL_CASES[case], cfg.cutoff[0])
    cr, ca = NO.maxneigh(fr, cfg.cutoff[0], cfg.cutoff[1])
    mr, ma = int(cr.max()) + 2, int(ca.max()) + 1
    exp = NO.neighbor(fr, cfg.cutoff[0], cfg.cutoff[1], mr, ma, with_rij)
    got = gpu_neighbor(fr, cfg, mr, ma, with_rij)
    assert_lists_equal(got, exp)


def _lattice_frames():
    """Perfect FCC crystals: many pair-vector components are exactly zero, which exercises the
    signed-zero handling of the orthorhombic path.  One with mirrored (-0.0) coordinates and
    one left-handed cell (negative first vector, so h^-1 has -0.0 off-diagonals)."""
    st = structures.fcc(3.615, (10, 10, 10), 0.0, seed=1)
    a = NP.frames_from_structures([st], 6.0)
    b = NP.frames_from_structures([st], 6.0)
    b.position = -b.position
    lat = np.diag([-36.15, 36.15, 36.15])
    box, bo, nc, _ = NP.expand_box(lat, 6.0)
    c = NP.NepFrames(st.frac @ lat, np.zeros(st.natoms, np.int64),
                     np.array([st.natoms]), box[None], bo[None], nc[None])
    return {"fcc": a, "fcc_mirrored": b, "fcc_left_handed": c}


@pytest.mark.parametrize("case", ["fcc", "fcc_mirrored", "fcc_left_handed"])
def test_neighbor_signed_zeros_match_oracle(case):
    fr = _lattice_frames()[case]
    cfg = NP.NepConfig(atom_type=[29])
    cr, ca = NO.maxneigh(fr, cfg.cutoff[0], cfg.cutoff[1])
    mr, ma = int(cr.max()), int(ca.max())
    exp = NO.neighbor(fr, cfg.cutoff[0], cfg.cutoff[1], mr, ma, True)
    got = gpu_neighbor(fr, cfg, mr, ma, True)
    assert_lists_equal(got, exp)


def test_maxneigh_matches_oracle():
    cfg = NP.NepConfig(atom_type=[3, 14, 8, 72])
    fr = _frames(CELL_CASES["mixed_batch"], cfg.cutoff[0])
    na, tm, bx, bo, nc, pos = _t(fr)
    for typed in (False, True):
        r, a = ops.calculate_maxneigh(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1],
                                      cfg.ntypes, tm, typed)
        er, ea = NO.maxneigh(fr, cfg.cutoff[0], cfg.cutoff[1], cfg.ntypes, typed)
        assert np.array_equal(r.cpu().numpy(), er) and np.array_equal(a.cpu().numpy(), ea)


def test_neighbor_overflow_is_reported():
    cfg = NP.NepConfig(atom_type=[3, 14, 8, 72])
    fr = _frames(CELL_CASES["cubic_1500"], cfg.cutoff[0])
    with pytest.raises(ops.NeighborOverflow):
        gpu_neighbor(fr, cfg, 20, 40)


def _exact_rows(fr, atoms, rc):
    """numpy restatement (IEEE double, no FMA) of the reference pair vector for a few atoms of a
    single num_cell = (1,1,1) frame: the expected (n2 ascending) lists."""
    pos, box, bo = fr.position, fr.box[0], fr.box_orig[0]
    dz = [(bo[3 * k] * 0.0 + bo[3 * k + 1] * 0.0) + bo[3 * k + 2] * 0.0 for k in range(3)]
    rows = []
    for n1 in atoms:
        d = [(pos[:, k] + dz[k]) - pos[n1, k] for k in range(3)]
        s = [((box[9 + 3 * k] * d[0] + box[10 + 3 * k] * d[1]) + box[11 + 3 * k] * d[2])
             for k in range(3)]
        s = [v - np.rint(v) for v in s]
        x = [((box[3 * k] * s[0] + box[3 * k + 1] * s[1]) + box[3 * k + 2] * s[2]) for k in range(3)]
        d2 = (x[0] * x[0] + x[1] * x[1]) + x[2] * x[2]
        keep = np.nonzero((d2 < rc * rc) & (np.arange(len(pos)) != n1))[0]
        rows.append((keep, np.stack([np.sqrt(d2[keep]), x[0][keep], x[1][keep], x[2][keep]], -1)))
    return rows


def test_neighbor_100k_properties():
    """100,000 atoms, four elements, density 0.06 (the NEP benchmark box): counts agree with
    calculate_maxneigh, rows are ascending, the lists are symmetric with exactly negated pair
    vectors, and sampled rows equal an IEEE-double numpy restatement."""
    cfg = NP.NepConfig(atom_type=[3, 14, 8, 72])
    st = structures.random_packed(100_000, 0.06, [3, 14, 8, 72], [0.25] * 4, seed=4)
    fr = NP.frames_from_structures([st], cfg.cutoff[0])
    na, tm, bx, bo, nc, pos = _t(fr)
    cr, ca = ops.calculate_maxneigh(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], 4, tm, False)
    mr, ma = int(cr.max()), int(ca.max())
    NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = ops.calculate_neighbor(
        na, tm, torch.arange(4, device=DEV), bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], mr, ma,
        True)
    assert torch.equal(NN_r, cr) and torch.equal(NN_a, ca)
    for NN, NL, Ri in ((NN_r, NL_r, Ri_r), (NN_a, NL_a, Ri_a)):
        S = NL.shape[1]
        slot = torch.arange(S, device=DEV).unsqueeze(0)
        valid = slot < NN.unsqueeze(1)
        assert torch.equal(NL >= 0, valid)
        big = torch.where(valid, NL, torch.full_like(NL, 1 << 40))
        assert bool(((big[:, 1:] > big[:, :-1]) | ~valid[:, 1:]).all())
        i = torch.arange(NL.shape[0], device=DEV).unsqueeze(1).expand_as(NL)[valid]
        j = NL[valid]
        fwd = torch.sort(i * 200_000 + j).values
        rev = torch.sort(j * 200_000 + i).values
        assert torch.equal(fwd, rev)
        # pair vector of (j, i) is the exact negation of (i, j)
        key_ij = i * 200_000 + j
        order = torch.argsort(key_ij)
        vec = Ri[valid][:, 1:][order]
        key_ji = j * 200_000 + i
        order2 = torch.argsort(key_ji)
        vec2 = Ri[valid][:, 1:][order2]
        assert torch.equal(vec, -vec2)
    rows = _exact_rows(fr, [0, 777, 54_321, 99_999], cfg.cutoff[0])
    NLc, Ric, NNc = NL_r.cpu().numpy(), Ri_r.cpu().numpy(), NN_r.cpu().numpy()
    for n1, (keep, vals) in zip([0, 777, 54_321, 99_999], rows):
        assert NNc[n1] == len(keep)
        assert np.array_equal(NLc[n1, :len(keep)], keep)
        assert np.array_equal(Ric[n1, :len(keep)].view(np.uint8), vals.view(np.uint8))


# ----------------------------------------------------------------------------------------------
# fused evaluation
# ----------------------------------------------------------------------------------------------
def _eval(c_cfg, params, lists, num_atom, type_map, precision):
    model = NP.NEP(c_cfg, params, precision=precision)
    t = lambda a: torch.as_tensor(a).to(DEV)  # noqa: E731
    NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = (t(x) for x in lists)
    Etot, Ei, F, _, V = model(NN_r, NL_r, Ri_r, NN_a, NL_a, Ri_a,
                              t(np.asarray(num_atom).reshape(-1, 1)), t(type_map))
    torch.cuda.synchronize()
    return (Etot.double().cpu().numpy(), Ei.double().cpu().numpy(), F.double().cpu().numpy(),
            V.double().cpu().numpy())


@pytest.mark.parametrize("name", CASES)
def test_eval_f64_matches_reference_fixture(nep_case, name):
    c = nep_case(name)
    g = c.g
    lists = (c.NN_r, c.NN_a, c.NL_r, c.NL_a, c.Ri_r, c.Ri_a)
    E, Ei, F, V = _eval(c.cfg, c.params, lists, g["num_atom"], g["type_map"], "float64")
    np.testing.assert_allclose(E.ravel(), g["Etot"].ravel(), rtol=1e-12)
    np.testing.assert_allclose(Ei, g["Ei"].reshape(-1), rtol=0, atol=1e-11 * np.abs(g["Ei"]).max())
    np.testing.assert_allclose(F, g["Force"], rtol=0, atol=1e-10 * np.abs(g["Force"]).max())
    np.testing.assert_allclose(V, g["Virial"], rtol=0, atol=1e-10 * np.abs(g["Virial"]).max())


@pytest.mark.parametrize("name", CASES)
def test_eval_f32_within_tolerance(nep_case, name):
    """FP32 form against the reference FP64 values: force error <= 1e-4 eV/A (RMSE and max <=
    5e-4), energy <= 1e-5 eV/atom."""
    c = nep_case(name)
    g = c.g
    lists = (c.NN_r, c.NN_a, c.NL_r, c.NL_a, c.Ri_r, c.Ri_a)
    E, Ei, F, V = _eval(c.cfg, c.params, lists, g["num_atom"], g["type_map"], "float32")
    n = g["num_atom"].reshape(-1)
    err_f = F - g["Force"]
    rmse = float(np.sqrt((err_f ** 2).mean()))
    print(f"[accuracy] nep {name} f32: force RMSE {rmse:.2e} max {np.abs(err_f).max():.2e} "
          f"E/atom {np.abs(E.ravel() - g['Etot'].ravel()).max() / n.max():.2e}")
    assert rmse <= 1e-4 and np.abs(err_f).max() <= 5e-4
    assert np.all(np.abs(E.ravel() - g["Etot"].ravel()) / n <= 1e-5)
    np.testing.assert_allclose(V, g["Virial"], rtol=0, atol=1e-4 * np.abs(g["Virial"]).max())


def test_eval_variants_match_oracle():
    """3-body only without the radial block, and a general-shape model (n_max 6, basis 12,
    wider net) through the compiled general kernel, FP64 against the oracle."""
    for cfg, seed in [
        (NP.NepConfig(atom_type=[3, 14, 8, 72], train_2b=False, l_max=(4, 2, 0)), 61),
        (NP.NepConfig(atom_type=[3, 14, 8, 72], n_max=(6, 5), basis_size=(12, 10), neuron=100), 62),
    ]:
        fr = _frames([(700, 0.06, seed, 0.02)], cfg.cutoff[0])
        cr, ca = NO.maxneigh(fr, cfg.cutoff[0], cfg.cutoff[1])
        lists = NO.neighbor(fr, cfg.cutoff[0], cfg.cutoff[1], int(cr.max()), int(ca.max()))
        p = NP.init_params(cfg, seed)
        o = NO.nep_eval(cfg, p, fr.num_atom, torch.tensor(fr.type_map), *(
            torch.tensor(x) for x in (lists[2], lists[4], lists[3], lists[5])), return_feats=True)
        p["q_scaler"] = NP.calc_q_scaler(cfg, o["feats"])
        o = NO.nep_eval(cfg, p, fr.num_atom, torch.tensor(fr.type_map), *(
            torch.tensor(x) for x in (lists[2], lists[4], lists[3], lists[5])))
        E, Ei, F, V = _eval(cfg, p, lists, fr.num_atom, fr.type_map, "float64")
        np.testing.assert_allclose(E.ravel(), o["Etot"].numpy().ravel(), rtol=1e-12)
        np.testing.assert_allclose(F, o["Force"].numpy(), rtol=0,
                                   atol=1e-10 * np.abs(o["Force"].numpy()).max())
        np.testing.assert_allclose(V, o["Virial"].numpy(), rtol=0,
                                   atol=1e-10 * np.abs(o["Virial"].numpy()).max())


def test_eval_batch_and_neighbor_chain_match_oracle():
    """GPU neighbor lists fed straight into the evaluator on a three-frame batch (cell-list and
    enumerated frames together), FP64 against the oracle."""
    cfg = NP.NepConfig(atom_type=[3, 14, 8, 72])
    fr = _frames(CELL_CASES["mixed_batch"], cfg.cutoff[0])
    cr, ca = NO.maxneigh(fr, cfg.cutoff[0], cfg.cutoff[1])
    mr, ma = int(cr.max()), int(ca.max())
    lists = gpu_neighbor(fr, cfg, mr, ma)
    p = NP.init_params(cfg, 71, energy_shift=-2.0)
    ex = NO.neighbor(fr, cfg.cutoff[0], cfg.cutoff[1], mr, ma)
    tt = lambda i: torch.tensor(ex[i])  # noqa: E731
    o = NO.nep_eval(cfg, p, fr.num_atom, torch.tensor(fr.type_map), tt(2), tt(4), tt(3), tt(5),
                    return_feats=True)
    p["q_scaler"] = NP.calc_q_scaler(cfg, o["feats"])
    o = NO.nep_eval(cfg, p, fr.num_atom, torch.tensor(fr.type_map), tt(2), tt(4), tt(3), tt(5))
    E, Ei, F, V = _eval(cfg, p, lists, fr.num_atom, fr.type_map, "float64")
    np.testing.assert_allclose(E.ravel(), o["Etot"].numpy().ravel(), rtol=1e-12)
    np.testing.assert_allclose(Ei, o["Ei"].numpy(), rtol=0, atol=1e-10)
    np.testing.assert_allclose(F, o["Force"].numpy(), rtol=0,
                               atol=1e-10 * np.abs(o["Force"].numpy()).max())
    np.testing.assert_allclose(V, o["Virial"].numpy(), rtol=0,
                               atol=1e-10 * np.abs(o["Virial"].numpy()).max())


def test_eval_forces_are_energy_gradient_on_gpu(nep_case):
    """Central differences of the GPU FP64 energy with the GPU neighbor lists rebuilt."""
    c = nep_case("nep_q4_240")
    g = c.g
    fr = NP.NepFrames(g["position"].copy(), g["type_map"], g["num_atom"], g["box"],
                      g["box_orig"], g["num_cell"])
    mr, ma = int(g["max_r"]), int(g["max_a"])
    lists = gpu_neighbor(fr, c.cfg, mr, ma)
    _, _, F, _ = _eval(c.cfg, c.params, lists, g["num_atom"], g["type_map"], "float64")
    h = 1e-5
    base = fr.position.copy()
    for atom, comp in [(5, 0), (100, 1), (239, 2)]:
        es = []
        for sgn in (1, -1):
            fr.position = base.copy()
            fr.position[atom, comp] += sgn * h
            ls = gpu_neighbor(fr, c.cfg, mr, ma)
            E, _, _, _ = _eval(c.cfg, c.params, ls, g["num_atom"], g["type_map"], "float64")
            es.append(float(E.sum()))
        fd = -(es[0] - es[1]) / (2 * h)
        assert abs(fd - F[atom, comp]) < 1e-6 * max(1.0, abs(fd))


def test_eval_bad_type_is_reported(nep_case):
    from matpl_gb300 import _lib
    c = nep_case("nep_hfo_l4")
    g = c.g
    tm = g["type_map"].copy()
    tm[7] = 5
    with pytest.raises(_lib.MatplError):
        _eval(c.cfg, c.params, (c.NN_r, c.NN_a, c.NL_r, c.NL_a, c.Ri_r, c.Ri_a), g["num_atom"],
              tm, "float32")


@pytest.mark.parametrize("name", CASES)
def test_descriptor_matches_reference_fixture(nep_case, name):
    """The q of NEP.calculate_qn (before q_scaler): FP64 to 1e-12, FP32 to 1e-5 relative."""
    c = nep_case(name)
    g = c.g
    t = lambda a: torch.as_tensor(a).to(DEV)  # noqa: E731
    NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = (t(x) for x in (c.NN_r, c.NN_a, c.NL_r, c.NL_a, c.Ri_r,
                                                         c.Ri_a))
    scale = np.abs(g["feats"]).max(0)
    for prec, tol in (("float64", 1e-12), ("float32", 1e-5)):
        m = NP.NEP(c.cfg, c.params, precision=prec)
        f = m.descriptor(NN_r, NL_r, Ri_r, NN_a, NL_a, Ri_a, t(g["num_atom"]), t(g["type_map"]))
        f = f.double().cpu().numpy()
        assert np.all(np.abs(f - g["feats"]) <= tol * scale), prec


def test_eval_zbl_matches_oracle_and_reference(nep_case):
    """The ZBL term (outer cutoff 2.2 A; pairs in the inner and the switching region, two
    frames).  FP64 = the oracle with the kernel's correctly rounded float32 element factors to
    1e-10 (E to 1e-12); = the reference's own values (golden) to 1e-7 relative: the reference's
    float32 Z^0.23 (torch pow) is one ulp off for some pairs; FP32 within 1e-5 of the force and
    virial scale."""
    c = nep_case("nep_zbl")
    g = c.g
    lists = (c.NN_r, c.NN_a, c.NL_r, c.NL_a, c.Ri_r, c.Ri_a)
    ref = NO.nep_eval(c.cfg, c.params, g["num_atom"], torch.tensor(g["type_map"]),
                      torch.tensor(c.NL_r), torch.tensor(c.Ri_r), torch.tensor(c.NL_a),
                      torch.tensor(c.Ri_a), zbl_factors="rounded")
    rE, rF, rV = ref["Etot"].numpy().ravel(), ref["Force"].numpy(), ref["Virial"].numpy()
    E, Ei, F, V = _eval(c.cfg, c.params, lists, g["num_atom"], g["type_map"], "float64")
    np.testing.assert_allclose(E.ravel(), rE, rtol=1e-12)
    np.testing.assert_allclose(Ei, ref["Ei"].numpy(), rtol=0, atol=1e-11 * np.abs(rE).max())
    np.testing.assert_allclose(F, rF, rtol=0, atol=1e-10 * np.abs(rF).max())
    np.testing.assert_allclose(V, rV, rtol=0, atol=1e-10 * np.abs(rV).max())
    np.testing.assert_allclose(E.ravel(), g["Etot"].ravel(), rtol=1e-7)
    np.testing.assert_allclose(F, g["Force"], rtol=0, atol=1e-7 * np.abs(g["Force"]).max())
    np.testing.assert_allclose(V, g["Virial"], rtol=0, atol=1e-7 * np.abs(g["Virial"]).max())
    E, Ei, F, V = _eval(c.cfg, c.params, lists, g["num_atom"], g["type_map"], "float32")
    print(f"[accuracy] nep zbl f32: force max err / max |F| "
          f"{np.abs(F - rF).max() / np.abs(rF).max():.2e}")
    np.testing.assert_allclose(E.ravel(), rE, rtol=1e-5)
    np.testing.assert_allclose(F, rF, rtol=0, atol=1e-5 * np.abs(rF).max())
    np.testing.assert_allclose(V, rV, rtol=0, atol=1e-5 * np.abs(rV).max())
