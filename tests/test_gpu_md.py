"""Batched replica MD: the CUDA-graph step equals the eager step, energies are conserved."""
import numpy as np
import pytest
import torch

from matpl_gb300 import md, params as P, structures
from oracle import neigh

pytestmark = pytest.mark.gpu


def _setup(precision, n_rep=(1, 2, 1), seed=3):
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
    cfg, prm, davg, dstd, reps = _setup("float64")
    a = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], dt_fs=1.0, precision="float64")
    b = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], dt_fs=1.0, precision="float64")
    assert len(a.groups) == 3 and a.nreplicas == 4
    a.step(5)
    for _ in range(5):
        b._step()
    torch.cuda.synchronize()
    a.check_errors()
    for ga, gb in zip(a.groups, b.groups):
        assert torch.allclose(ga["x"], gb["x"], rtol=0, atol=1e-11)
        assert torch.allclose(ga["v"], gb["v"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(a.energies(), b.energies(), rtol=1e-11)


@pytest.mark.parametrize("precision,tol", [("float64", 2e-5), ("mixed", 2e-4)])
def test_energy_is_conserved(precision, tol):
    """Velocity Verlet, dt = 0.5 fs, 200 steps: |E(t) - E(0)| per atom stays small."""
    cfg, prm, davg, dstd, reps = _setup(precision)
    sim = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], dt_fs=0.5, precision=precision)
    e0 = sim.energies().sum(1)
    n = sim.natoms()
    worst = 0.0
    for _ in range(20):
        sim.step(10)
        e = sim.energies().sum(1)
        worst = max(worst, float(np.max(np.abs(e - e0) / n)))
    sim.check_errors()
    print(f"[accuracy] MD {precision}: max |E(t)-E(0)| per atom over 200 steps {worst:.2e} eV")
    assert worst < tol
