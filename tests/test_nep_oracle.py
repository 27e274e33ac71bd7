"""Pin the NEP oracle against golden vectors produced by MatPL's own NEP code (the reference's
CPU neighbor operator built from its sources, and ``nep_net.NEP``'s CPU branch)."""
import hashlib

import numpy as np
import pytest
import torch

from matpl_gb300 import nep as NP
from oracle import nep_oracle as NO

CASES = ["nep_q4_240", "nep_q4_tri2", "nep_hfo_l4", "nep_zbl"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_expand_box_matches_fixture(nep_case):
    for name in CASES:
        c = nep_case(name)
        g = c.g
        for b in range(g["lattice"].shape[0]):
            box, bo, nc, _ = NP.expand_box(g["lattice"][b], float(g["cutoff"][0]))
            assert np.array_equal(box, g["box"][b])
            assert np.array_equal(bo, g["box_orig"][b])
            assert np.array_equal(nc, g["num_cell"][b])


@pytest.mark.parametrize("name", CASES)
def test_oracle_neighbor_bit_exact(nep_case, name):
    c = nep_case(name)
    g = c.g
    NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = NO.neighbor(c.frames, c.cfg.cutoff[0], c.cfg.cutoff[1],
                                                     int(g["max_r"]), int(g["max_a"]))
    assert np.array_equal(NN_r, g["NN_r"]) and np.array_equal(NN_a, g["NN_a"])
    assert _sha(NL_r) == str(g["sha_NL_r"]) and _sha(NL_a) == str(g["sha_NL_a"])
    assert _sha(Ri_r) == str(g["sha_Ri_r"]) and _sha(Ri_a) == str(g["sha_Ri_a"])
    cr, ca = NO.maxneigh(c.frames, c.cfg.cutoff[0], c.cfg.cutoff[1])
    assert np.array_equal(cr, g["cnt_r"]) and np.array_equal(ca, g["cnt_a"])
    tr, ta = NO.maxneigh(c.frames, c.cfg.cutoff[0], c.cfg.cutoff[1], c.cfg.ntypes, True)
    assert np.array_equal(tr.reshape(-1, c.cfg.ntypes).sum(1), cr)
    assert np.array_equal(ta.reshape(-1, c.cfg.ntypes).sum(1), ca)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_nep(nep_case, name):
    c = nep_case(name)
    g = c.g
    out = NO.nep_eval(c.cfg, c.params, g["num_atom"], torch.tensor(g["type_map"]),
                      torch.tensor(c.NL_r), torch.tensor(c.Ri_r), torch.tensor(c.NL_a),
                      torch.tensor(c.Ri_a), return_feats=True)
    np.testing.assert_allclose(out["feats"].numpy(), g["feats"], rtol=1e-12,
                               atol=1e-12 * np.abs(g["feats"]).max())
    np.testing.assert_allclose(out["Etot"].numpy().ravel(), g["Etot"].ravel(), rtol=1e-12)
    np.testing.assert_allclose(out["Ei"].numpy(), g["Ei"].reshape(-1), rtol=0,
                               atol=1e-11 * np.abs(g["Ei"]).max())
    np.testing.assert_allclose(out["Force"].numpy(), g["Force"], rtol=0,
                               atol=1e-11 * np.abs(g["Force"]).max())
    np.testing.assert_allclose(out["Virial"].numpy(), g["Virial"], rtol=0,
                               atol=1e-11 * np.abs(g["Virial"]).max())


def test_q_scaler_restatement(nep_case):
    for name in CASES:
        c = nep_case(name)
        qs = NP.calc_q_scaler(c.cfg, torch.tensor(c.g["feats"]))
        np.testing.assert_allclose(qs.numpy(), c.g["q_scaler"], rtol=1e-14)


def test_oracle_forces_are_energy_gradient(nep_case):
    """Independent of the reference: central differences of Etot with the neighbor lists
    rebuilt at every displaced position."""
    c = nep_case("nep_q4_tri2")
    g = c.g
    fr = c.frames
    base = fr.position.copy()
    out = NO.nep_eval(c.cfg, c.params, g["num_atom"], torch.tensor(g["type_map"]),
                      torch.tensor(c.NL_r), torch.tensor(c.Ri_r), torch.tensor(c.NL_a),
                      torch.tensor(c.Ri_a))
    h = 1e-5
    for atom, comp in [(3, 0), (17, 2), (50, 1)]:
        es = []
        for sgn in (1, -1):
            fr.position = base.copy()
            fr.position[atom, comp] += sgn * h
            _, _, NLr, NLa, Rr, Ra = NO.neighbor(fr, c.cfg.cutoff[0], c.cfg.cutoff[1],
                                                 int(g["max_r"]), int(g["max_a"]))
            o = NO.nep_eval(c.cfg, c.params, g["num_atom"], torch.tensor(g["type_map"]),
                            torch.tensor(NLr), torch.tensor(Rr), torch.tensor(NLa), torch.tensor(Ra))
            es.append(float(o["Etot"].sum()))
        fd = -(es[0] - es[1]) / (2 * h)
        assert abs(fd - float(out["Force"][atom, comp])) < 1e-6 * max(1.0, abs(fd))
    fr.position = base


def test_zbl_rounded_factors_close_to_reference(nep_case):
    """The oracle's "rounded" ZBL element factors (the kernel's: correctly rounded float32
    Z^0.23) against the reference's own values (torch's float32 pow): within 1e-7 relative."""
    c = nep_case("nep_zbl")
    g = c.g
    out = NO.nep_eval(c.cfg, c.params, g["num_atom"], torch.tensor(g["type_map"]),
                      torch.tensor(c.NL_r), torch.tensor(c.Ri_r), torch.tensor(c.NL_a),
                      torch.tensor(c.Ri_a), zbl_factors="rounded")
    np.testing.assert_allclose(out["Etot"].numpy().ravel(), g["Etot"].ravel(), rtol=1e-7)
    np.testing.assert_allclose(out["Force"].numpy(), g["Force"], rtol=0,
                               atol=1e-7 * np.abs(g["Force"]).max())
    # the ZBL term is what moves these frames: without it the energies differ entirely
    import dataclasses
    off = NO.nep_eval(dataclasses.replace(c.cfg, zbl=None), c.params, g["num_atom"],
                      torch.tensor(g["type_map"]), torch.tensor(c.NL_r), torch.tensor(c.Ri_r),
                      torch.tensor(c.NL_a), torch.tensor(c.Ri_a))
    assert np.abs(off["Etot"].numpy().ravel() - g["Etot"].ravel()).min() > 1.0
