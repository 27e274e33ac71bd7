"""Batched replica MD on the ragged skin-list step.

* The CUDA-graph step equals the eager step.
* The forces of the skin-filtered list equal those of a fresh exact search (the drop-in
  ``find_neighbore``) at the same moved positions, replica by replica, also after rebuilds that
  a small skin forces.
* Energy is conserved.
"""
import numpy as np
import pytest
import torch

from matpl_gb300 import dp, md, ops, params as P, structures
from oracle import neigh

pytestmark = pytest.mark.gpu


def _setup(n_rep=(1, 2, 1), seed=3):
    cfg = P.DPConfig(atom_type=[29], maxNeighborNum=100, Rmax=6.0, Rmin=0.5)
    sizes = [(2, 2, 2), (3, 3, 3), (2, 3, 4)]
    reps = []
    for k, (r, c) in enumerate(zip(sizes, n_rep)):
        for q in range(c):
            reps.append(structures.fcc(3.615, r, 0.05, seed=seed + 10 * k + q))
    st = structures.fcc(3.615, (3, 3, 3), 0.05, seed=1)
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 1, 100, 6.0, [6.0])
    davg, dstd = P.calc_stat(cfg, ln, idr, st.types)
    prm = P.init_params(cfg, 101)
    return cfg, prm, davg, dstd, reps


def test_graph_step_equals_eager_step():
    cfg, prm, davg, dstd, reps = _setup()
    a = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], dt_fs=1.0, precision="float64",
                     steps_per_graph=5)
    b = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], dt_fs=1.0, precision="float64")
    assert a.nreplicas == 4 and a.natoms_total == sum(r.natoms for r in reps)
    a.step(10)
    for _ in range(10):
        b._step()
    torch.cuda.synchronize()
    a.check_errors()
    assert torch.allclose(a.x, b.x, rtol=0, atol=1e-11)
    assert torch.allclose(a.v, b.v, rtol=0, atol=1e-12)
    np.testing.assert_allclose(a.energies(), b.energies(), rtol=1e-11)


def _exact_forces(cfg, prm, davg, dstd, sim, r, precision):
    """Forces of replica r from the drop-in search at the simulation's current positions."""
    sl = sim.replica_slice(r)
    x = sim.x[sl].double()
    lat = sim.lat[r]
    frac = torch.remainder(x @ sim.inv_lat[r], 1.0)
    frac = torch.where(frac >= 1.0, torch.zeros_like(frac), frac)
    m = dp.DP(cfg, prm, davg, dstd, precision=precision, device=sim.dev)
    ln, idr = ops.find_neighbore(sim.types[sl], frac.contiguous(), lat, 1, 100, 6.0, 6.0,
                                 out_dtype=m.dtype)
    out = m.evaluate(ln, sim.types[sl], m.present_types(cfg.atom_type), idr, 0)
    return out["Force"][0].double(), out["Ei_atom"][0].double()


@pytest.mark.parametrize("precision,skin,tol", [("float64", 1.0, 1e-10), ("float64", 0.02, 1e-10),
                                                ("mixed", 1.0, 2e-5)])
def test_skin_list_forces_equal_a_fresh_exact_search(precision, skin, tol):
    cfg, prm, davg, dstd, reps = _setup()
    sim = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], dt_fs=2.0, temperature_k=600.0,
                       precision=precision, skin=skin)
    sim.step(12)
    torch.cuda.synchronize()
    sim.check_errors()
    nb = sim.rebuilds()
    if skin < 0.1:
        assert nb > 2, nb             # the small skin forces rebuilds during the run
    else:
        assert nb >= 1, nb
    F = sim.out["Force"][0].double()
    Ei = sim.out["Ei_atom"][0].double()
    for r in range(sim.nreplicas):
        sl = sim.replica_slice(r)
        Fx, Ex = _exact_forces(cfg, prm, davg, dstd, sim, r, precision)
        scale = max(1.0, float(Fx.abs().max()))
        assert float((F[sl] - Fx).abs().max()) <= tol * scale, r
        assert float((Ei[sl] - Ex).abs().max()) <= tol * max(1.0, float(Ex.abs().max())), r
    # the per-replica potential energy is the sum of that replica's atomic energies
    pe = sim.energies()[:, 0]
    for r in range(sim.nreplicas):
        assert abs(pe[r] - float(Ei[sim.replica_slice(r)].sum())) <= 1e-9 * max(1.0, abs(pe[r]))


@pytest.mark.parametrize("precision,tol", [("float64", 2e-5), ("mixed", 2e-4)])
def test_energy_is_conserved(precision, tol):
    """Velocity Verlet, dt = 0.5 fs, 200 steps: |E(t) - E(0)| per atom stays small."""
    cfg, prm, davg, dstd, reps = _setup()
    sim = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], dt_fs=0.5, precision=precision,
                       steps_per_graph=10)
    e0 = sim.energies().sum(1)
    n = sim.natoms()
    worst = 0.0
    for _ in range(20):
        sim.step(10)
        e = sim.energies().sum(1)
        worst = max(worst, float(np.max(np.abs(e - e0) / n)))
    sim.check_errors()
    print(f"[accuracy] MD {precision}: max |E(t)-E(0)| per atom over 200 steps {worst:.2e} eV, "
          f"{sim.rebuilds()} list builds")
    assert worst < tol


def test_two_element_replicas_match_exact_search():
    """Li / Si replicas of different sizes (two type blocks per atom): after a few steps the
    skin-filtered list gives the forces of a fresh exact search, replica by replica (FP64)."""
    cfg = P.DPConfig(atom_type=[3, 14], maxNeighborNum=150, Rmax=6.0, Rmin=0.5)
    reps = [structures.random_packed(n, 0.05, [3, 14], [0.5, 0.5], seed=40 + k)
            for k, n in enumerate((90, 140, 64))]
    st = reps[1]
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, 150, 6.0, [6.0, 6.0])
    davg, dstd = P.calc_stat(cfg, ln, idr, st.types)
    prm = P.init_params(cfg, 7)
    sim = md.ReplicaMD(cfg, prm, davg, dstd, reps, [6.94, 28.086], dt_fs=1.0,
                       precision="float64", skin=0.3)
    sim.step(6)
    torch.cuda.synchronize()
    sim.check_errors()
    F = sim.out["Force"][0]
    for r in range(sim.nreplicas):
        sl = sim.replica_slice(r)
        x = sim.x[sl]
        frac = torch.remainder(x @ sim.inv_lat[r], 1.0)
        frac = torch.where(frac >= 1.0, torch.zeros_like(frac), frac)
        m = dp.DP(cfg, prm, davg, dstd, precision="float64", device=sim.dev)
        l2, i2 = ops.find_neighbore(sim.types[sl], frac.contiguous(), sim.lat[r], 2, 150, 6.0, 6.0)
        Fx = m.evaluate(l2, sim.types[sl], m.present_types(cfg.atom_type), i2, 0)["Force"][0]
        scale = max(1.0, float(Fx.abs().max()))
        assert float((F[sl] - Fx).abs().max()) <= 1e-10 * scale, r


def test_skin_list_overflow_is_reported():
    """A skin-list capacity below what the cells need: the build flags a neighbor overflow
    (no write past the list) and check_errors raises."""
    cfg, prm, davg, dstd, reps = _setup()
    sim = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], precision="float64",
                       skin_capacity=40)
    torch.cuda.synchronize()
    with pytest.raises(Exception, match="error code 1"):
        sim.check_errors()
