"""NEP Verlet-skin lists (ops.SkinNeighbor): at every call the lists equal calculate_neighbor's at
the same positions bit for bit, whether the skin list was rebuilt or only filtered; rebuilds
follow the skin / 2 displacement rule; the compact MD form (int32 / f32, FP32 pair vectors from
the build plus displacements) has the same pairs with vectors within a few FP32 ulps and gives
the same forces to FP32 accuracy; a captured step (move + lists + fused evaluation) replays like
the eager one."""
import numpy as np
import pytest
import torch

from matpl_gb300 import nep as NP, ops, structures

pytestmark = pytest.mark.gpu
DEV = "cuda"
ELEMS = [3, 14, 8, 72]


def _frames(specs, cutoff):
    sts = [structures.random_packed(n, d, ELEMS, [0.25] * 4, seed=s, strain=e)
           for (n, d, s, e) in specs]
    return NP.frames_from_structures(sts, cutoff)


def _t(fr):
    c = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=DEV)  # noqa: E731
    return (c(fr.num_atom.reshape(-1, 1), torch.int64), c(fr.type_map, torch.int64),
            c(fr.box, torch.float64), c(fr.box_orig, torch.float64),
            c(fr.num_cell, torch.int64), c(fr.position, torch.float64))


def _exact(cfg, na, tm, bx, bo, nc, pos, mr, ma, with_rij=True):
    at = torch.arange(cfg.ntypes, device=DEV)
    return ops.calculate_neighbor(na, tm, at, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1],
                                  mr, ma, with_rij)


def _assert_same(got, exp, what):
    names = ["NN_r", "NN_a", "NL_r", "NL_a", "Ri_r", "Ri_a"]
    for n, g, e in zip(names, got, exp):
        assert g.shape == e.shape, (what, n)
        if g.dtype == torch.float64:
            g, e = g.view(torch.int64), e.view(torch.int64)
        if not torch.equal(g, e):
            bad = (g != e).nonzero()[:5].tolist()
            raise AssertionError(f"{what}: {n} differs at {bad}")


def _random_moves(n, max_len, gen):
    d = torch.randn(n, 3, generator=gen, dtype=torch.float64)
    d = d / d.norm(dim=1, keepdim=True)
    return (d * max_len * torch.rand(n, 1, generator=gen, dtype=torch.float64)).to(DEV)


CASES = {
    "cubic_3000": [(3000, 0.06, 61, 0.0)],
    "tri_3000": [(3000, 0.06, 62, 0.05)],
    "two_frames": [(2000, 0.06, 63, 0.02), (2600, 0.07, 64, 0.0)],
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("with_rij", [True, False])
def test_skin_lists_equal_the_exact_search(case, with_rij):
    cfg = NP.NepConfig(atom_type=ELEMS)
    fr = _frames(CASES[case], cfg.cutoff[0])
    na, tm, bx, bo, nc, pos = _t(fr)
    zeros = torch.zeros_like(tm)
    cr, ca = ops.calculate_maxneigh(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], 1,
                                    zeros, False)
    mr, ma = int(cr.max()) + 12, int(ca.max()) + 8     # room for the moves below
    sk = ops.SkinNeighbor(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], mr, ma,
                          with_rij=with_rij, skin=1.0)
    _assert_same(sk.lists(pos), _exact(cfg, na, tm, bx, bo, nc, pos, mr, ma, with_rij), "p0")
    assert sk.rebuilds() == 1
    gen = torch.Generator().manual_seed(7)
    N = pos.shape[0]
    # every atom moves up to 0.45 A (< skin / 2) from the build positions: no rebuild, pairs
    # that came up to 0.9 A closer are found in the skin list
    p1 = pos + _random_moves(N, 0.45, gen)
    _assert_same(sk.lists(p1), _exact(cfg, na, tm, bx, bo, nc, p1, mr, ma, with_rij), "p1")
    assert sk.rebuilds() == 1
    # a few atoms now beyond skin / 2 from the build positions: rebuild
    p2 = p1.clone()
    p2[::97] = pos[::97] + _random_moves(p2[::97].shape[0], 0.05, gen) + 0.6 / 3 ** 0.5
    _assert_same(sk.lists(p2), _exact(cfg, na, tm, bx, bo, nc, p2, mr, ma, with_rij), "p2")
    assert sk.rebuilds() == 2
    # atoms carried out of the cell by a lattice vector (unwrapped coordinates) and a random
    # walk of small steps afterwards
    p3 = p2.clone()
    lat = bo.reshape(-1, 3, 3).transpose(1, 2)[0]          # rows = lattice vectors (frame 0)
    n0 = int(fr.num_atom[0])
    p3[: n0: 5] += lat[0] - lat[2]
    p = p3
    for k in range(12):
        _assert_same(sk.lists(p), _exact(cfg, na, tm, bx, bo, nc, p, mr, ma, with_rij),
                     f"walk {k}")
        p = p + _random_moves(N, 0.12, gen)
    nb = sk.rebuilds()
    assert 3 <= nb < 3 + 12     # the wrap rebuilds once; the walk rebuilds now and then
    sk.check_errors()


def _assert_compact_close(got, exp, rc, what):
    """Compact lists against the exact ones: same counts and indices (a pair within 1e-5 A of a
    cutoff may differ), vectors within a few FP32 ulps."""
    for rad, (nn_g, nl_g, ri_g, nn_e, nl_e, ri_e) in enumerate(
            [(got[0], got[2], got[4], exp[0], exp[2], exp[4]),
             (got[1], got[3], got[5], exp[1], exp[3], exp[5])]):
        cut = rc[rad]
        nn_g, nn_e = nn_g.long(), nn_e.long()
        bad = (nn_g != nn_e).nonzero().flatten().tolist()
        for i in bad:      # only pairs at the cutoff may move across it
            a = set(nl_g[i, :nn_g[i]].tolist()) ^ set(nl_e[i, :nn_e[i]].tolist())
            r = ri_e[i, :nn_e[i], 0].double()
            near = (r - cut).abs() < 1e-5
            assert len(a) == 1 and (near.any() or nn_g[i] > nn_e[i]), (what, i, a)
        ok = (nn_g == nn_e)
        m = int(nn_e.max())
        slots = torch.arange(m, device=nn_e.device)[None, :] < nn_e[:, None]
        mask = slots & ok[:, None]
        assert torch.equal(nl_g[:, :m].long()[mask], nl_e[:, :m][mask]), what
        d = (ri_g[:, :m].double() - ri_e[:, :m])[mask].abs().max()
        assert float(d) < 3e-6, (what, float(d))


@pytest.mark.parametrize("case", ["cubic_3000", "two_frames"])
def test_compact_skin_lists_match_the_exact_search(case):
    cfg = NP.NepConfig(atom_type=ELEMS)
    fr = _frames(CASES[case], cfg.cutoff[0])
    na, tm, bx, bo, nc, pos = _t(fr)
    zeros = torch.zeros_like(tm)
    cr, ca = ops.calculate_maxneigh(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], 1,
                                    zeros, False)
    mr, ma = int(cr.max()) + 12, int(ca.max()) + 8
    sk = ops.SkinNeighbor(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], mr, ma,
                          compact=True)
    gen = torch.Generator().manual_seed(9)
    N = pos.shape[0]
    p = pos
    for k in range(10):
        L = sk.lists(p)
        assert L[2].dtype == torch.int32 and L[4].dtype == torch.float32
        _assert_compact_close(L, _exact(cfg, na, tm, bx, bo, nc, p, mr, ma), cfg.cutoff,
                              f"step {k}")
        p = p + _random_moves(N, 0.2, gen)
    assert 2 <= sk.rebuilds() < 10
    sk.check_errors()


def test_compact_lists_give_the_forces_of_the_exact_lists():
    cfg = NP.NepConfig(atom_type=ELEMS)
    fr = _frames([(4000, 0.06, 68, 0.03)], cfg.cutoff[0])
    na, tm, bx, bo, nc, pos = _t(fr)
    prm = NP.init_params(cfg, 6, energy_shift=-3.0)
    m32 = NP.NEP(cfg, prm, "float32", device=DEV)
    m64 = NP.NEP(cfg, prm, "float64", device=DEV)
    zeros = torch.zeros_like(tm)
    cr, ca = ops.calculate_maxneigh(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], 1,
                                    zeros, False)
    mr, ma = int(cr.max()) + 12, int(ca.max()) + 8
    sk = ops.SkinNeighbor(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], mr, ma,
                          compact=True)
    p = pos + _random_moves(pos.shape[0], 0.4, torch.Generator().manual_seed(3))
    L = sk.lists(p)
    assert sk.rebuilds() == 1          # the filter of the first build's list
    E = _exact(cfg, na, tm, bx, bo, nc, p, mr, ma)
    rc = m32.evaluate(L[0], L[2], L[4], L[1], L[3], L[5], na, tm)
    r32 = m32.evaluate(E[0], E[2], E[4], E[1], E[3], E[5], na, tm)
    r64 = m64.evaluate(E[0], E[2], E[4], E[1], E[3], E[5], na, tm)
    F64 = r64["Force"]
    err_c = float((rc["Force"].double() - F64).abs().max())
    err_e = float((r32["Force"].double() - F64).abs().max())
    scale = float(F64.abs().max())
    assert err_c <= 4 * err_e + 1e-7 * scale, (err_c, err_e, scale)
    assert abs(float(rc["Etot"]) - float(r64["Etot"])) <= 1e-6 * pos.shape[0]
    verr_c = float((rc["Virial"] - r64["Virial"]).abs().max())
    verr_e = float((r32["Virial"] - r64["Virial"]).abs().max())
    assert verr_c <= 4 * verr_e + 1e-7 * float(r64["Virial"].abs().max()), (verr_c, verr_e)


def test_skin_overflow_and_thin_boxes_are_reported():
    cfg = NP.NepConfig(atom_type=ELEMS)
    fr = _frames([(3000, 0.06, 65, 0.0)], cfg.cutoff[0])
    na, tm, bx, bo, nc, pos = _t(fr)
    with pytest.raises(ops.NeighborOverflow):
        ops.SkinNeighbor(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], 200, 100,
                         capacity=20)
    with pytest.raises(ops.NeighborOverflow):
        ops.SkinNeighbor(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], 10, 100)
    small = _frames([(60, 0.06, 66, 0.0)], cfg.cutoff[0])
    with pytest.raises(ValueError):
        ops.SkinNeighbor(*[t for i, t in enumerate(_t(small)) if i != 1], cfg.cutoff[0],
                         cfg.cutoff[1], 200, 100)


@pytest.mark.parametrize("compact", [False, True])
def test_skin_step_in_a_cuda_graph_replays_like_eager(compact):
    cfg = NP.NepConfig(atom_type=ELEMS)
    fr = _frames([(4000, 0.06, 67, 0.03)], cfg.cutoff[0])
    na, tm, bx, bo, nc, pos0 = _t(fr)
    prm = NP.init_params(cfg, 5, energy_shift=-3.0)
    model = NP.NEP(cfg, prm, "float32", device=DEV, check_errors=False)
    zeros = torch.zeros_like(tm)
    cr, ca = ops.calculate_maxneigh(na, bx, bo, nc, pos0, cfg.cutoff[0], cfg.cutoff[1], 1,
                                    zeros, False)
    mr, ma = int(cr.max()) + 12, int(ca.max()) + 8
    N = pos0.shape[0]
    vel = _random_moves(N, 0.04, torch.Generator().manual_seed(11))

    def make():
        pos = pos0.clone()
        sk = ops.SkinNeighbor(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], mr, ma,
                              compact=compact)
        return pos, sk

    def step(pos, sk):
        pos.add_(vel)
        L = sk.lists(pos)
        return model.evaluate(L[0], L[2], L[4], L[1], L[3], L[5], na, tm)

    pos_e, sk_e = make()
    eager = []
    for _ in range(25):
        r = step(pos_e, sk_e)
        eager.append((r["Force"].clone(), r["Etot"].clone()))
    pos_g, sk_g = make()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        step(pos_g, sk_g)                        # warm-up on the side stream (workspaces)
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        out = step(pos_g, sk_g)
    # the captured step has not run yet; the warm-up moved the atoms once
    graphed = [(eager[0][0], eager[0][1])]
    for _ in range(24):
        g.replay()
        graphed.append((out["Force"].clone(), out["Etot"].clone()))
    torch.cuda.synchronize()
    for k, ((fe, ee), (fg, eg)) in enumerate(zip(eager, graphed)):
        scale = float(fe.abs().max())
        assert torch.allclose(fg, fe, rtol=0, atol=2e-6 * scale), k
        assert abs(float(eg) - float(ee)) <= 1e-9 * abs(float(ee)) + 1e-9, k
    assert torch.equal(pos_g, pos_e)
    assert sk_g.rebuilds() == sk_e.rebuilds() >= 2    # 25 x 0.04 A moves: at least one rebuild
    sk_g.check_errors()
