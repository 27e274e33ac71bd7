"""GPU neighbor search vs the oracle restatement of NeighConst.f90: bit-exact index lists
and dR, both branches (periodic images / nearest image), triclinic cells, batches, overflow."""
import numpy as np
import pytest
import torch

from matpl_gb300 import ops, structures
from oracle import neigh

pytestmark = pytest.mark.gpu
DEV = "cuda"


def gpu_build(st, ntypes, m, rc=6.0, rct=None, out_dtype=torch.float64, lat=None, frac=None):
    lat = st.lattice if lat is None else lat
    frac = st.frac if frac is None else frac
    return ops.find_neighbore(torch.tensor(st.types), torch.tensor(frac, device=DEV),
                              torch.tensor(lat), ntypes, m, rc, rct if rct is not None else rc,
                              out_dtype=out_dtype)


def assert_same(st, ntypes, m, rc=6.0, rct=None):
    ln_o, idr_o = neigh.find_neighbore(st.types, st.frac, st.lattice, ntypes, m, rc,
                                       rct if rct is not None else [rc] * ntypes)
    ln_g, idr_g = gpu_build(st, ntypes, m, rc, rct)
    assert np.array_equal(ln_g.cpu().numpy(), ln_o)
    assert np.array_equal(idr_g.cpu().numpy(), idr_o)   # bitwise, including r = sqrt(dd)
    return ln_o


@pytest.mark.parametrize("name", ["cu108_f64", "lisi600_f64", "hfo48_f64", "hfo2_jit"])
def test_golden_structures_bit_exact(golden_case, name):
    c = golden_case(name)
    g = c.g
    for b in range(g["lattice"].shape[0]):
        st = structures.Structure(g["lattice"][b], g["frac"][b], c.types, list(c.cfg.atom_type))
        ln = assert_same(st, c.cfg.ntypes, c.cfg.maxNeighborNum, c.cfg.Rmax)
        assert np.array_equal(ln, c.list_neigh[b:b + 1])


def test_large_box_cell_list_bit_exact():
    st = structures.random_packed(4000, 0.05, [3, 14], [0.5, 0.5], seed=9)
    assert_same(st, 2, 150)


def test_triclinic_skewed_nearest_image_branch():
    st = structures.random_packed(3000, 0.07, [72, 8], [1 / 3, 2 / 3], seed=4, strain=0.03)
    L = st.lattice.copy()
    L[1] += 0.3 * L[0]          # strong shear: thickness < lattice vector length
    st = structures.Structure(L, st.frac, st.types, st.elements)
    assert_same(st, 2, 200)


def test_per_type_cutoff_and_float32_output():
    st = structures.random_packed(500, 0.06, [1, 2, 3], [0.3, 0.3, 0.4], seed=2)
    assert_same(st, 3, 120, rc=6.0, rct=[5.0, 6.0, 5.5])
    ln_o, idr_o = neigh.find_neighbore(st.types, st.frac, st.lattice, 3, 120, 6.0, [6.0] * 3)
    ln_g, idr_g = gpu_build(st, 3, 120, out_dtype=torch.float32)
    assert np.array_equal(ln_g.cpu().numpy(), ln_o)
    assert np.array_equal(idr_g.cpu().numpy(), idr_o.astype(np.float32))


def test_batch_of_images_matches_per_image_calls():
    sts = [structures.fcc(3.615, (3, 3, 3), 0.05, seed=s) for s in range(3)]
    lat = np.stack([s.lattice for s in sts])
    frac = np.stack([s.frac for s in sts])
    ln_g, idr_g = ops.find_neighbore(torch.tensor(sts[0].types), torch.tensor(frac, device=DEV),
                                     torch.tensor(lat), 1, 100, 6.0, 6.0)
    for b, s in enumerate(sts):
        ln_o, idr_o = neigh.find_neighbore(s.types, s.frac, s.lattice, 1, 100, 6.0, [6.0])
        assert np.array_equal(ln_g[b:b + 1].cpu().numpy(), ln_o)
        assert np.array_equal(idr_g[b:b + 1].cpu().numpy(), idr_o)


def test_overflow_raises():
    st = structures.fcc(3.615, (3, 3, 3), 0.05, seed=11)
    with pytest.raises(ops.NeighborOverflow):
        gpu_build(st, 1, 50)
    st2 = structures.random_packed(3000, 0.05, [3, 14], [0.5, 0.5], seed=1)
    with pytest.raises(ops.NeighborOverflow):
        gpu_build(st2, 2, 20)


def test_tiny_and_empty_inputs():
    st = structures.Structure(np.eye(3) * 20.0, np.array([[0.1, 0.1, 0.1], [0.15, 0.1, 0.1]]),
                              np.array([0, 0], dtype=np.int32), [1])
    assert_same(st, 1, 10)
    one = structures.Structure(np.eye(3) * 3.0, np.array([[0.5, 0.5, 0.5]]),
                               np.array([0], dtype=np.int32), [1])
    assert_same(one, 1, 200)   # periodic self images count as neighbors


def test_full_size_counts_and_symmetry():
    """32k-atom Li/Si box (m = 150 per type): every pair appears in both lists with opposite
    dR (nearest-image branch, equal cutoffs) and the counts match the oracle's."""
    st = structures.random_packed(32000, 0.05, [3, 14], [0.5, 0.5], seed=2024)
    ln_g, idr_g, cnt = ops.find_neighbore(torch.tensor(st.types), torch.tensor(st.frac, device=DEV),
                                          torch.tensor(st.lattice), 2, 150, 6.0, 6.0,
                                          with_counts=True)
    ln = ln_g[0].long()
    assert int(cnt.max()) <= 150
    n_tot = int((ln > 0).sum())
    assert 40 * 32000 < n_tot < 52 * 32000
    i_idx = torch.arange(32000, device=DEV).unsqueeze(1).expand_as(ln)
    mask = ln > 0
    pairs_fwd = (i_idx[mask] * 32000 + (ln[mask] - 1)).sort().values
    pairs_rev = ((ln[mask] - 1) * 32000 + i_idx[mask]).sort().values
    assert torch.equal(pairs_fwd, pairs_rev)


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.int64 if a.dtype == np.float64 else np.int32)


@pytest.mark.parametrize("variant", ["plain", "neg_zero", "neg_diag"])
def test_orthorhombic_crystal_exact_zeros_bitwise(variant):
    """A perfect FCC crystal (non-cubic orthorhombic cell) in the nearest-image branch: many
    pair components are exact zeros, so the signed-zero handling of the orthorhombic form must
    give the general formula's bits (compared as integers, so -0.0 != +0.0): off-diagonal zeros
    +0.0 or -0.0, and a negative diagonal entry (left-handed cell) that turns products of +0
    into -0."""
    st = structures.fcc(3.615, (6, 5, 7), 0.0, seed=1)
    L = st.lattice.copy()
    if variant == "neg_zero":
        for q in ((0, 1), (0, 2), (1, 0), (1, 2), (2, 0), (2, 1)):
            L[q] = -0.0
    if variant == "neg_diag":
        L[0, 0] = -L[0, 0]
        L[1, 0] = -0.0
    st = structures.Structure(L, st.frac, st.types, st.elements)
    ln_o, idr_o = neigh.find_neighbore(st.types, st.frac, st.lattice, 1, 100, 6.0, [6.0])
    for dt, ref in ((torch.float64, idr_o), (torch.float32, idr_o.astype(np.float32))):
        ln_g, idr_g = gpu_build(st, 1, 100, out_dtype=dt)
        assert np.array_equal(ln_g.cpu().numpy(), ln_o)
        assert np.array_equal(_bits(idr_g.cpu().numpy()), _bits(ref))
    assert (idr_o[..., 1:] == 0).any()
