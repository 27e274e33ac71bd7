"""Pin the oracle against the golden vectors produced by MatPL's own DP implementation."""
import hashlib

import numpy as np
import pytest
import torch

from oracle import dp_oracle, neigh

CASES = ["cu108_f64", "cu108_f32", "cu108x2_f64", "lisi600_f64", "hfo48_f64", "hfo2_jit"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", CASES)
def test_oracle_neighbor_list_is_stable(golden_case, name):
    c = golden_case(name)
    assert _sha(c.list_neigh) == str(c.g["list_sha"])
    assert _sha(c.image_dr) == str(c.g["imagedr_sha"])
    assert np.array_equal((c.list_neigh > 0).sum(-1), c.g["nneigh"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_dp(golden_case, name):
    c = golden_case(name)
    g = c.g
    dt = c.dtype
    p = {k: v.to(dt) for k, v in c.params.items()}
    out = dp_oracle.dp_eval(c.cfg, p, c.davg, c.dstd, torch.tensor(c.list_neigh),
                            torch.tensor(c.types), torch.tensor(c.cfg.atom_type),
                            torch.tensor(c.image_dr, dtype=dt), 0)
    rtol = 1e-10 if dt == torch.float64 else 2e-4
    np.testing.assert_allclose(out["Etot"].detach().numpy().ravel(), g["Etot"].ravel(), rtol=rtol)
    np.testing.assert_allclose(out["Ei"].detach().numpy(), g["Ei"].reshape(out["Ei"].shape),
                               rtol=rtol, atol=rtol * np.abs(g["Ei"]).max())
    fs = np.abs(g["Force"]).max()
    np.testing.assert_allclose(out["Force"].detach().numpy(), g["Force"], rtol=0, atol=rtol * fs * 10)
    vs = np.abs(g["Virial"]).max()
    np.testing.assert_allclose(out["Virial"].detach().numpy(), g["Virial"], rtol=0, atol=rtol * vs * 10)
    if "dE" in g:
        np.testing.assert_allclose(out["dE"].detach().numpy(), g["dE"], rtol=0,
                                   atol=1e-12 * np.abs(g["dE"]).max())


def test_op_oracle_reproduces_reference_scatter(golden_case):
    """The calculateForce/calculateVirial oracle, fed the reference's own dE, gives the
    reference's forces (dp_dp.py:436-459 and CalcOps.cpp:6-22 agree)."""
    c = golden_case("cu108_f64")
    g = c.g
    ln = torch.tensor(c.list_neigh)
    idr = torch.tensor(c.image_dr)
    Ri, Ri_d = dp_oracle.env_matrix(c.cfg, idr, torch.tensor(c.types), c.davg, c.dstd)
    dE = torch.tensor(g["dE"])
    B, N, S = ln.shape
    Rd = Ri_d.reshape(B, N, 4 * S, 3)
    Fc = -(dE.reshape(B, N, 1, 4 * S) @ Rd).squeeze(-2)
    F, V, AV = dp_oracle.force_virial_ops(ln - 1, dE.reshape(B, N, 4 * S), Rd, idr[..., 1:], Fc, 0)
    np.testing.assert_allclose(F.numpy(), g["Force"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(V.numpy(), g["Virial"], rtol=0, atol=1e-10 * np.abs(g["Virial"]).max())


def test_neighbor_overflow_raises():
    from matpl_gb300 import structures
    cu = structures.fcc(3.615, (3, 3, 3), 0.05, seed=11)
    with pytest.raises(neigh.NeighborOverflow):
        neigh.find_neighbore(cu.types, cu.frac, cu.lattice, 1, 50, 6.0, [6.0])


def test_neighbor_sets_match_bruteforce_numpy():
    """Independent check of the restatement: the set of (i, j, |r|) within Rc equals an
    all-images numpy enumeration for a skewed small cell (periodic-image branch)."""
    from matpl_gb300 import structures
    st = structures.random_packed(40, 0.07, [72, 8], [1 / 3, 2 / 3], seed=5, strain=0.03)
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, 200, 6.0, [6.0, 6.0])
    lat = st.lattice
    frac = np.mod(st.frac + 10.0, 1.0)
    n = len(st.types)
    npd = [int(6.0 / np.linalg.norm(lat[v])) + 1 for v in range(3)]
    for i in range(n):
        got = sorted((int(ln[0, i, s]) - 1, round(float(idr[0, i, s, 0]), 9))
                     for s in range(ln.shape[2]) if ln[0, i, s] > 0)
        exp = []
        for j in range(n):
            for a in range(-npd[0], npd[0] + 1):
                for b in range(-npd[1], npd[1] + 1):
                    for cc in range(-npd[2], npd[2] + 1):
                        d = (frac[j] - frac[i] + np.array([a, b, cc])) @ lat
                        dd = float(d @ d)
                        if 1e-8 < dd < 36.0:
                            exp.append((j, round(np.sqrt(dd), 9)))
        assert got == sorted(exp)


def test_compress_oracle_matches_reference_cpu_formula():
    """The reference's CPU branch (dp_dp.py:590-597) writes the order-5 polynomial term by term;
    the oracle's G must agree with that expression and its derivative with finite differences."""
    g = torch.Generator().manual_seed(0)
    f2 = torch.rand(50, 1, generator=g, dtype=torch.float64)
    c = torch.randn(50, 25, 6, generator=g, dtype=torch.float64)
    G, dG = dp_oracle.compress_oracle(f2, c)
    ref = (f2 ** 5 * c[:, :, 0] + f2 ** 4 * c[:, :, 1] + f2 ** 3 * c[:, :, 2] + f2 ** 2 * c[:, :, 3]
           + f2 * c[:, :, 4] + c[:, :, 5])
    assert torch.allclose(G, ref, rtol=1e-14, atol=1e-14)
    h = 1e-6
    Gp, _ = dp_oracle.compress_oracle(f2 + h, c)
    Gm, _ = dp_oracle.compress_oracle(f2 - h, c)
    assert torch.allclose((Gp - Gm) / (2 * h), dG, rtol=1e-6, atol=1e-6)


def test_chunked_oracle_equals_the_whole_evaluation(golden_case):
    """dp_eval_chunked (the oracle the 32k-atom parity test uses) = dp_eval on the pinned
    600-atom Li/Si case, with chunks that split both element groups."""
    c = golden_case("lisi600_f64")
    args = (c.cfg, c.params, c.davg, c.dstd, torch.tensor(c.list_neigh), torch.tensor(c.types),
            torch.tensor(c.cfg.atom_type), torch.tensor(c.image_dr))
    whole = dp_oracle.dp_eval(*args, 0, virial_convention="gpu")
    part = dp_oracle.dp_eval_chunked(*args, chunk=97)
    assert abs(part["Etot"].item() - whole["Etot"].item()) <= 1e-12 * abs(whole["Etot"].item())
    for k in ("Ei_atom", "Force", "Virial"):
        scale = whole[k].abs().max().item()
        assert (part[k] - whole[k].detach()).abs().max().item() <= 1e-12 * scale, k
    np.testing.assert_allclose(part["Etot"].numpy().ravel(), c.g["Etot"].ravel(), rtol=1e-10)
