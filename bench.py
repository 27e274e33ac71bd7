"""Benchmark: DP se_e2_a energy + force + virial throughput (atom-steps/s) on GB300.

Workload (the headline configuration): 32,000 atoms, Li:Si 1:1, random-packed periodic cube at
0.05 atoms/A^3 (minimum pair distance 2.0 A, seeded), Rc = 6.0 A, Rmin = 0.5 A, 150 neighbor
slots per type (S = 300); embedding 1->25->25->25, M2 = 16, fitting 400->50->50->50->1, random
weights W ~ N(0, 1/fan_in).  One step = neighbor search from fractional positions + energy,
forces and virial (what an MD step needs).  Synthetic data: no dataset is involved.

  value : step with inputs resident in HBM (per-step working set ~230 MB > 129 MB L2), in the
          mixed-precision form (tcgen05 BF16x3 GEMMs); the plain-FP32 form of the same step is
          timed in the same run and reported beside it (config.plain_fp32, speedup)
  e2e   : the same step through the public API with host (pinned) positions copied in and
          energy / forces / virial copied out every step
  roofline : the dominant kernel, timed live with CUDA events on its stream
  cpu_baseline : MatPL's DP algorithm (oracle port of dp_dp_script.DP, torch FP64) on the
          host cores, on a bounded 4,000-atom sample of the same workload

A second workload, NEP (100,000 atoms, four elements, radial / angular cutoffs 6 / 4 A), is
measured in the same run and reported in the line's "nep" object (step = calculate_neighbor with
exact FP64 lists + the fused FP32 energy / force / virial kernel); --workload nep prints it as
its own line.  Further objects: "train" (force-loss training step), "md" (batched replica MD)
and "lammps" (the headline box as LAMMPS hands it to pair_style matpl: local + ghost atoms and a
full list in random order, one PairMATPL.compute per step from host arrays to host forces;
--workload lammps prints it as its own line).

--impl reference runs only the CPU implementation (oracle port) and prints its line.
For N > 1 (torchrun) every rank runs its own replica (replicas only, weak scaling).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

NATOMS, DENSITY, M_NEIGH, RC, RMIN = 32000, 0.05, 150, 6.0, 0.5
ELEMENTS = [3, 14]
SEED_STRUCT, SEED_W = 2024, 11
METRIC = "E+F+virial atom-steps/s, mixed vs plain FP32 at force err ≤1e-4 eV/Å"
CPU_SAMPLE = 4000

# algorithmic FLOPs (no recompute): per occupied pair of the embedding forward / backward and
# per atom of the fitting part (25 -> 25 -> 25 embedding, M2 = 16, 400 -> 50 -> 50 -> 50 -> 1)
FLOP_EMB_FWD_PAIR = 2 * (25 + 625 + 625) + 2 * 4 * 25          # 2750
FLOP_EMB_BWD_PAIR = 2 * 2 * 100 + 2 * (625 + 625 + 25) + 42     # 2992
FLOP_FIT_ATOM = 2 * 4 * 25 * 16 + 2 * 2 * (400 * 50 + 50 * 50 + 50 * 50 + 50) + 2 * 3200


# NEP workload: 100,000 atoms, four elements in equal parts, 0.06 atoms/A^3 random-packed cube;
# radial cutoff 6 A (basis 8 -> 9 functions, n_max 4), angular cutoff 4 A (basis 8, n_max 4,
# l_max 4 / 2 / 1), one 30-unit tanh hidden layer per element, seeded random parameters
NEP_NATOMS, NEP_DENSITY, NEP_ELEMENTS = 100_000, 0.06, [3, 14, 8, 72]
NEP_SEED_STRUCT, NEP_SEED_W = 2025, 12
NEP_CPU_SAMPLE = 4000
NEP_METRIC = "NEP E+F+virial atom-steps/s, fused FP32 vs FP64 oracle"


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:                       # host-only ranks (the multi-process tests): gloo
            dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    """The largest of every rank's x (the slowest replica sets the time of a step)."""
    if ws == 1:
        return x
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def replica_value(units_per_rank, ms_max, ws):
    """Whole-job throughput of ws replicas: the units all ranks processed / the step time of
    the slowest rank (ms, already reduced by max_over_ranks)."""
    return ws * units_per_rank / (ms_max * 1e-3)


def sm_count() -> int:
    """Streaming multiprocessors of the current GPU (the SIMT peak is quoted per SM)."""
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def make_workload(natoms=NATOMS, seed=SEED_STRUCT):
    from matpl_gb300 import params as P, structures
    st = structures.random_packed(natoms, DENSITY, ELEMENTS, [0.5, 0.5], seed=seed)
    cfg = P.DPConfig(atom_type=list(ELEMENTS), maxNeighborNum=M_NEIGH, Rmax=RC, Rmin=RMIN)
    prm = P.init_params(cfg, SEED_W)
    return st, cfg, prm


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index
        out_dir = os.environ.get("MATPL_BENCH_OUT", tempfile.gettempdir())
        self.path = os.path.join(out_dir, f"clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.gpu)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = [l.split(",") for l in open(self.path).read().splitlines() if l.strip()]
        sm, mx, pw, reasons = [], None, [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1])); mx = float(r[2]); pw.append(float(r[3]))
                for k, n in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "power_w_max": max(pw) if pw else None, "samples": len(sm),
                "reasons": sorted(reasons)}


def cpu_baseline_run(steps, warmup):
    """MatPL's DP algorithm on the host cores (oracle port), bounded 4,000-atom sample."""
    from oracle import dp_oracle, neigh
    from matpl_gb300 import params as P
    ncores = os.cpu_count() or 1
    torch.set_num_threads(ncores)
    st, cfg, prm = make_workload(CPU_SAMPLE, seed=SEED_STRUCT + 1)
    ln, idr = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, M_NEIGH, RC, [RC, RC])
    davg, dstd = P.calc_stat(cfg, ln, idr, st.types)
    args = (cfg, prm, torch.tensor(davg), torch.tensor(dstd))
    at = torch.tensor(cfg.atom_type)
    tm = torch.tensor(st.types)

    def step():
        l, r = neigh.find_neighbore(st.types, st.frac, st.lattice, 2, M_NEIGH, RC, [RC, RC])
        out = dp_oracle.dp_eval(*args, torch.tensor(l), tm, at, torch.tensor(r), 0)
        return out["Etot"].item()

    for _ in range(warmup):
        step()
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        step()
        ts.append(time.perf_counter() - t0)
    med = statistics.median(ts)
    return {"value": CPU_SAMPLE / med, "unit": "atom-steps/s", "cores": ncores, "kind": "port",
            "sample": f"{CPU_SAMPLE}-atom Li/Si box of the same density, m=150/type, FP64, "
                      f"neighbor search + E/F/V per step, median of {steps}",
            "sec_per_step": med, "steps": steps}


def nep_flops(cfg, n_r_pairs, n_a_pairs, natoms):
    """Algorithmic FLOPs of one NEP E+F+V evaluation (no recompute), from the model shape:
    per radial pair   basis f_k and f_k' (6 kr), g_n and g_n' (4 nr kr), dE/dr (2 nr), force
                      and virial (24);
    per angular pair  basis (6 ka), g_n and g_n' (4 na ka), 24 harmonics (40), s_nlm (48 na),
                      adjoint sums A_n and B_lm (96 na), harmonic gradients (80), G (144),
                      force and virial (38);
    per atom          features (48 na + 30 na), network forward 2 F H + H and adjoint
                      2 F H + F + 5 H, dE/ds (10 * 24 na)."""
    nr, kr, na, ka, F, H = cfg.nr, cfg.kr, cfg.na, cfg.ka, cfg.feature_nums, cfg.neuron
    pr = 6 * kr + 4 * nr * kr + 2 * nr + 24
    pa = 6 * ka + 4 * na * ka + 40 + 48 * na + 96 * na + 80 + 144 + 38
    at = 78 * na + 2 * F * H + H + 2 * F * H + F + 5 * H + 240 * na
    return pr * n_r_pairs + pa * n_a_pairs + at * natoms


def nep_workload(natoms=NEP_NATOMS, seed=NEP_SEED_STRUCT):
    from matpl_gb300 import nep as NP, structures
    cfg = NP.NepConfig(atom_type=list(NEP_ELEMENTS))
    st = structures.random_packed(natoms, NEP_DENSITY, NEP_ELEMENTS, [0.25] * 4, seed=seed)
    fr = NP.frames_from_structures([st], cfg.cutoff[0])
    prm = NP.init_params(cfg, NEP_SEED_W, energy_shift=-3.0)
    return cfg, fr, prm, st


def cpu_baseline_nep(steps, warmup):
    """MatPL's NEP algorithm on the host cores: the oracle port (restated neighbor operator in C,
    nep_net.NEP's CPU descriptor / network / autograd forces in torch FP64) on a bounded sample."""
    from oracle import nep_oracle as NO
    ncores = os.cpu_count() or 1
    torch.set_num_threads(ncores)
    cfg, fr, prm, _ = nep_workload(NEP_CPU_SAMPLE, seed=NEP_SEED_STRUCT + 1)
    cr, ca = NO.maxneigh(fr, cfg.cutoff[0], cfg.cutoff[1])
    mr, ma = int(cr.max()), int(ca.max())
    tm = torch.tensor(fr.type_map)

    def step():
        L = NO.neighbor(fr, cfg.cutoff[0], cfg.cutoff[1], mr, ma)
        out = NO.nep_eval(cfg, prm, fr.num_atom, tm, torch.tensor(L[2]), torch.tensor(L[4]),
                          torch.tensor(L[3]), torch.tensor(L[5]))
        return float(out["Etot"].sum())

    for _ in range(warmup):
        step()
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        step()
        ts.append(time.perf_counter() - t0)
    med = statistics.median(ts)
    return {"value": NEP_CPU_SAMPLE / med, "unit": "atom-steps/s", "cores": ncores, "kind": "port",
            "sample": f"{NEP_CPU_SAMPLE}-atom four-element box of the same density and model, FP64, "
                      f"neighbor lists + E/F/V per step, median of {steps}",
            "sec_per_step": med, "steps": steps}


def nep_reference_gpu(cfg, prm, st, r32, r64, ours_ms, ours_e2e_ms, ours_eval_ms, mr, ma,
                      calls=10):
    """The reference's own GPU NEP evaluator on the same structure and model: the LAMMPS
    NEP3::compute_large_box_optim (nep3.cu:551-810), built unmodified for sm_103a from a staged
    copy of its sources (baseline/ref_gpu.py), reading a nep5 file written from the same
    parameters, on the LAMMPS view of the box (local atoms, ghost images within the largest
    cutoff + 1 A skin, full lists), driven as PairMATPL::compute drives it
    (pair_matpl.cpp:1093-1190).  Its call is synchronous: host positions in (plus type and list
    arrays on a rebuild step), host energies / forces / virial out."""
    try:
        from baseline import ref_gpu
    except ImportError as e:
        return {"unavailable": f"comparator module not importable: {e}"}
    from matpl_gb300 import lammps as L, nep as NP
    if ref_gpu.load() is None:
        return {"unavailable": "comparator library not built (reference GPU sources not staged)"}
    s = L.lammps_system(st.lattice, st.frac @ st.lattice, st.types + 1,
                        max(cfg.cutoff) + LMP_SKIN, seed=NEP_SEED_STRUCT)
    ref = ref_gpu.RefNEP(NP.gpumd_text(cfg, prm, (mr, ma)), s, s["type"] - 1,
                         device=torch.cuda.current_device())
    try:
        ei, f, v = ref.compute(True)
        n = s["nlocal"]
        F = L.fold_ghosts(f, s["owner"], n)
        F64 = r64["Force"].reshape(-1, 3).double().cpu().numpy()
        F32 = r32["Force"].reshape(-1, 3).double().cpu().numpy()
        V64 = r64["Virial"].reshape(-1)[[0, 4, 8, 1, 2, 5]].double().cpu().numpy()
        E64 = float(r64["Etot"].sum())
        parity = {"force_max_abs_err_vs_f64_eV_per_A": float(np.abs(F - F64).max()),
                  "force_rmse_vs_f64_eV_per_A": float(np.sqrt(((F - F64) ** 2).mean())),
                  "ours_f32_force_max_abs_err_vs_f64_eV_per_A": float(np.abs(F32 - F64).max()),
                  "energy_err_per_atom_eV": abs(float(ei.sum()) - E64) / n,
                  "virial_max_abs_err_eV": float(np.abs(v - V64).max())}

        def per_call(build, k):
            ref.compute(build)
            t0 = time.perf_counter()
            for _ in range(k):
                ref.compute(build)
            return (time.perf_counter() - t0) * 1e3 / k

        call_ms = per_call(False, calls)
        call_build_ms = per_call(True, max(3, calls // 2))
    finally:
        ref.close()
    # kernel-only times of both sides from one ncu launch list of this workload (committed)
    kern = None
    kp = os.path.join(HERE, "profiles", "reference_gpu_kernels.json")
    if os.path.exists(kp):
        kern = json.load(open(kp)).get("nep_100k")
    out = {"source": "src/lmps/lammps-libtorch/MATPL/NEP_GPU (nep3.cu, nep3_large_box.cuh), "
                     "unmodified, nvcc -O3 sm_103a",
           "system": {"nlocal": n, "nghost": s["nghost"], "max_listed": int(s["numneigh"].max()),
                      "list_capacity": ref.capacity, "max_pairs_in_cutoffs": ref.max_pairs},
           "call_ms": call_ms, "call_rebuild_ms": call_build_ms,
           "ours_step_ms": ours_ms, "ours_nep_eval_ms": ours_eval_ms, "ours_e2e_ms": ours_e2e_ms,
           "e2e_speedup": call_ms / ours_e2e_ms,
           "e2e_note": "reference call (host positions in, lists already on the GPU, E/F/V out) "
                       "vs our end-to-end step, which also rebuilds the exact lists every step",
           **parity}
    if kern and n == NEP_NATOMS:
        out["kernels_from_ncu"] = {
            "reference_us_per_call": kern["reference_total_us"],
            "ours_us_per_step": kern["ours_total_us"],
            "device_speedup": kern["reference_total_us"] / kern["ours_total_us"],
            "evaluation_speedup": kern["reference_evaluation_us"] / kern["ours_evaluation_us"],
            "source": "profiles/reference_gpu_kernels.json (cold, serialised launches of one ncu "
                      "launch list; device_speedup: its kernels per call - list filter + sort, "
                      "descriptor, forces, virial - against our whole step including the exact "
                      "list build; evaluation_speedup: its evaluation kernels against nep_eval)"}
    return out


NEP_MD_MASSES = {3: 6.94, 14: 28.085, 8: 15.999, 72: 178.49}   # amu, by atomic number
NEP_MD_STEPS = 60


def nep_skin_md(cfg, model, st, na, tm, bx, bo, nc, pos0, mr, ma, compact, steps=NEP_MD_STEPS):
    """The NEP step as an MD caller runs it: positions advance by v dt every step (Maxwell-
    Boltzmann velocities at 300 K, dt 1 fs; the forces are not fed back, so the atoms follow the
    motion of the first femtoseconds of an MD run without its integrator), the lists come from
    ops.SkinNeighbor (skin 1 A, rebuilt on the device when an atom has moved more than 0.5 A) and
    the fused FP32 evaluation; the whole step is one CUDA-graph replay.  ``compact``: the MD list
    form (FP32 pair vectors from the build plus displacements, int32 / f32 lists read by
    matpl_nep_eval_compact); otherwise lists bit-identical to calculate_neighbor's.  Timed over
    ``steps`` consecutive steps, so rebuild steps count at the rate the motion causes them."""
    from matpl_gb300 import _lib, ops, structures
    dev = pos0.device
    masses = np.array([NEP_MD_MASSES[NEP_ELEMENTS[t]] for t in st.types])
    vel = torch.tensor(structures.maxwell_boltzmann(masses, 300.0, seed=NEP_SEED_STRUCT),
                       dtype=torch.float64, device=dev)
    pos = pos0.clone()
    sk = ops.SkinNeighbor(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], mr + 8, ma + 6,
                          skin=1.0, compact=compact)

    def step():
        pos.add_(vel)                      # dt = 1 fs, v in A / fs
        L = sk.lists(pos)
        return model.evaluate(L[0], L[2], L[4], L[1], L[3], L[5], na, tm)

    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        for _ in range(3):
            step()
    torch.cuda.current_stream(dev).wait_stream(side)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        out = step()
    torch.cuda.synchronize()
    sk.check_errors()
    b0 = sk.rebuilds()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    nbuild = sk.rebuilds() - b0
    sk.check_errors()
    # per-kernel split from an eager, event-bracketed run of the same motion
    _lib.profile_begin(4096)
    b1 = sk.rebuilds()
    for _ in range(steps):
        step()
    torch.cuda.synchronize()
    prof = _lib.profile_collect()
    nb_prof = sk.rebuilds() - b1
    split = {k: {"ms_per_launch": v[0] / v[1], "launches": v[1]} for k, v in prof.items()}
    # the lists of the last step against the exact search at the same positions
    at = torch.arange(cfg.ntypes, device=dev)
    L = sk.lists(pos)
    E = ops.calculate_neighbor(na, tm, at, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1],
                               mr + 8, ma + 6, True)
    if compact:
        nn_same = bool(torch.equal(L[0].long(), E[0]) and torch.equal(L[1].long(), E[1]))
        slots = torch.arange(mr + 8, device=dev)[None, :] < E[0][:, None]
        vec_err = float((L[4].double() - E[4])[slots].abs().max())
        check = {"counts_equal_exact_search": nn_same,
                 "max_abs_pair_vector_err_A": vec_err}
        r = model.evaluate(L[0], L[2], L[4], L[1], L[3], L[5], na, tm)
        rx = model.evaluate(E[0], E[2], E[4], E[1], E[3], E[5], na, tm)
        check["max_abs_force_diff_vs_exact_lists_eV_per_A"] = float(
            (r["Force"] - rx["Force"]).abs().max())
    else:
        check = {"lists_equal_exact_search_bitwise": all(
            torch.equal(x.view(torch.int64) if x.dtype == torch.float64 else x,
                        y.view(torch.int64) if y.dtype == torch.float64 else y)
            for x, y in zip(L, E))}
    vmax = float(vel.norm(dim=1).max())
    del g, out
    return {"ms_per_step": ms, "value": pos0.shape[0] / (ms * 1e-3), "unit": "atom-steps/s",
            "steps_timed": steps, "rebuilds_in_timed_steps": nbuild,
            "rebuilds_in_profiled_steps": nb_prof, "skin_A": 1.0,
            "skin_capacity": sk.cap, "max_speed_A_per_fs": vmax, **check, "kernels": split,
            "list_form": "compact (int32 / f32, FP32 pair vectors)" if compact else
                         "calculate_neighbor's, bit-identical",
            "note": "MD-style caller: Verlet-skin lists (ops.SkinNeighbor) + fused FP32 E/F/V, "
                    "one CUDA-graph replay per step, positions advanced by v dt each step (300 K "
                    "Maxwell-Boltzmann, 1 fs); the drop-in step above rebuilds the exact lists "
                    "every step"}


def run_nep(args, ws, local, steps, warmup, sample_clocks=True):
    """The NEP step on this GPU: calculate_neighbor (exact FP64 lists, the reference's layout) +
    the fused FP32 descriptor / network / force / virial kernel, 100,000 atoms."""
    from matpl_gb300 import _lib, nep as NP, ops
    dev = torch.device("cuda", local)
    cfg, fr, prm, st = nep_workload(args.nep_atoms)
    N = fr.natoms
    c = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)  # noqa: E731
    na, tm, bx, bo, nc = (c(fr.num_atom.reshape(-1, 1), torch.int64), c(fr.type_map, torch.int64),
                          c(fr.box, torch.float64), c(fr.box_orig, torch.float64),
                          c(fr.num_cell, torch.int64))
    pos_d = c(fr.position, torch.float64)
    at = torch.arange(cfg.ntypes, device=dev)
    cr, ca = ops.calculate_maxneigh(na, bx, bo, nc, pos_d, cfg.cutoff[0], cfg.cutoff[1],
                                    cfg.ntypes, tm, False)
    mr, ma = int(cr.max()), int(ca.max())
    n_r, n_a = int(cr.sum()), int(ca.sum())
    lists = ops.calculate_neighbor(na, tm, at, bx, bo, nc, pos_d, cfg.cutoff[0], cfg.cutoff[1],
                                   mr, ma, True)
    # q_scaler from this box's descriptors (update_scaler_values, nep_net.py:1020-1058)
    m64 = NP.NEP(cfg, prm, "float64", device=dev)
    feats = m64.descriptor(lists[0], lists[2], lists[4], lists[1], lists[3], lists[5], na, tm)
    prm = dict(prm)
    prm["q_scaler"] = NP.calc_q_scaler(cfg, feats).cpu()
    m64 = NP.NEP(cfg, prm, "float64", device=dev)
    m32 = NP.NEP(cfg, prm, "float32", device=dev, check_errors=False)
    r64 = m64.evaluate(lists[0], lists[2], lists[4], lists[1], lists[3], lists[5], na, tm)

    def step(pos):
        NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a = ops.calculate_neighbor(
            na, tm, at, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], mr, ma, True,
            check_overflow=False)
        return m32.evaluate(NN_r, NL_r, Ri_r, NN_a, NL_a, Ri_a, na, tm)

    r32 = step(pos_d)
    torch.cuda.synchronize()
    acc = {"force_rmse_vs_f64_eV_per_A": (r32["Force"].double() - r64["Force"]).pow(2).mean().sqrt().item(),
           "force_max_abs_err_eV_per_A": (r32["Force"].double() - r64["Force"]).abs().max().item(),
           "energy_err_per_atom_eV": abs(r32["Etot"].item() - r64["Etot"].item()) / N,
           "virial_max_abs_err_eV": (r32["Virial"] - r64["Virial"]).abs().max().item()}
    for _ in range(warmup):
        step(pos_d)
    sampler = ClockSampler(local) if sample_clocks else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    _lib.profile_begin(max(4096, steps * 8))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step(pos_d)
    e1.record()
    torch.cuda.synchronize()
    prof = _lib.profile_collect()
    barrier(ws)
    clocks = sampler.stop() if sampler else None
    ms = max_over_ranks(e0.elapsed_time(e1) / steps, ws)

    # end to end: host positions in, energy / forces / virial out
    pos_h = torch.tensor(fr.position).pin_memory()
    F_h = torch.empty(N, 3, dtype=torch.float32).pin_memory()
    E_h = torch.empty(1, dtype=torch.float64).pin_memory()
    V_h = torch.empty(1, 9, dtype=torch.float64).pin_memory()

    def e2e_step():
        r = step(pos_h.to(dev, non_blocking=True))
        F_h.copy_(r["Force"], non_blocking=True)
        E_h.copy_(r["Etot"], non_blocking=True)
        V_h.copy_(r["Virial"], non_blocking=True)
        torch.cuda.current_stream().synchronize()

    for _ in range(3):
        e2e_step()
    e2e_steps = max(5, steps // 2)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    t1 = time.perf_counter()
    e2e_ms = max_over_ranks((t1 - t0) * 1e3 / e2e_steps, ws)

    per_kernel = {k: {"ms_per_launch": v[0] / v[1], "launches": v[1]} for k, v in prof.items()}
    tot = sum(v[0] for v in prof.values())
    for k, v in prof.items():
        per_kernel[k]["share"] = v[0] / tot if tot else None
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    simt_peak = sm_count() * 128 * 2 * sm_mhz * 1e6 / 1e12
    fl = nep_flops(cfg, n_r, n_a, N)
    t_eval = per_kernel["nep_eval"]["ms_per_launch"] * 1e-3
    # neighbor operator: reads positions (24 B / atom), writes NN (16 B / atom) and the padded
    # lists NL int64 + Ri f64 x 4 (40 B per slot, max_NN slots per atom, both lists)
    nb_bytes = N * (24 + 16 + 40 * (mr + ma))
    t_nb = per_kernel["nep_neighbor"]["ms_per_launch"] * 1e-3
    peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(HERE, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    # the eval kernel reads, per occupied slot, NL int64 + Ri f64 x 4 (40 B), per atom
    # type + two counts (24 B) and writes Ei, the force accumulator and force (32 B)
    ev_bytes = 40 * (n_r + n_a) + 56 * N
    launches = sum(v[1] for v in prof.values())
    traffic = None
    tp = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tp):
        tr = json.load(open(tp)).get("nep_eval:float32")
        if tr:   # recorded for the 100,000-atom launch; DRAM bytes scale with atoms
            traffic = {"bytes_per_launch": tr["bytes_per_launch"] * N / NEP_NATOMS,
                       "note": tr.get("note")}
    md_skin = nep_skin_md(cfg, m32, st, na, tm, bx, bo, nc, pos_d, mr, ma, compact=True)
    md_skin["exact_lists"] = nep_skin_md(cfg, m32, st, na, tm, bx, bo, nc, pos_d, mr, ma,
                                         compact=False)
    ref_gpu = None if args.no_ref_gpu else nep_reference_gpu(
        cfg, prm, st, r32, r64, ms, e2e_ms, per_kernel["nep_eval"]["ms_per_launch"], mr, ma)
    return {
        "metric": NEP_METRIC, "value": ws * N / (ms * 1e-3), "unit": "atom-steps/s",
        "ms_per_step": ms, "steps": steps, "warmup": warmup, "dtype": "f32 (f64 lists, f64 sums)",
        "config": {"workload": f"NEP, {N:,} atoms, 4 elements (equal parts) random-packed at "
                               "0.06 atoms/A^3; radial rc 6 A basis 8 n_max 4, angular rc 4 A "
                               "basis 8 n_max 4 l_max 4/2/1, 30-unit tanh layer per element; "
                               "step = calculate_neighbor + fused E/F/V",
                   "natoms": N, "radial_pairs": n_r, "angular_pairs": n_a,
                   "max_NN_radial": mr, "max_NN_angular": ma,
                   "l2": "no flush: per-step lists ~0.4 GB exceed the 129 MB L2", **acc},
        "e2e": {"value": ws * N / (e2e_ms * 1e-3), "unit": "atom-steps/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": pos_h.numel() * 8,
                "d2h_bytes_per_step": F_h.numel() * 4 + 8 + 72},
        "gpu_launches": launches, "kernels": per_kernel,
        "roofline": {"kernel": "nep_eval", "bound": "simt_fp32", "achieved": fl / t_eval / 1e12,
                     "peak": simt_peak, "unit": "TFLOP/s", "frac": fl / t_eval / 1e12 / simt_peak,
                     "algorithmic_flops_per_launch": fl,
                     "traffic": traffic["bytes_per_launch"] if traffic else None,
                     "traffic_note": traffic["note"] if traffic else None,
                     "peak_source": f"nominal FP32 SIMT at the sampled SM clock ({sm_count()} SMs x 128 lanes x 2)",
                     "hbm": {"achieved": ev_bytes / t_eval / 1e9, "peak": hbm_peak,
                             "unit": "GB/s", "frac": ev_bytes / t_eval / 1e9 / hbm_peak,
                             "algorithmic_bytes_per_launch": ev_bytes}},
        "reference_gpu": ref_gpu,
        "md_skin": md_skin,
        "neighbor_roofline": {"kernel": "nep_neighbor", "bound": "fp64 (exact reference arithmetic)",
                              "hbm_achieved": nb_bytes / t_nb / 1e9, "hbm_peak": hbm_peak,
                              "unit": "GB/s", "frac": nb_bytes / t_nb / 1e9 / hbm_peak,
                              "algorithmic_bytes_per_launch": nb_bytes},
        "clocks": clocks,
    }


TRAIN_METRIC = "DP force-loss training step atom-steps/s, fused vs plain FP32"
# force-loss training batch: 64 Hf:O (1:2) configurations with atom counts drawn uniformly in
# [32, 512], random-packed at 0.07 atoms/A^3 with a 3 % symmetric cell strain, the headline's
# nets (m = 100 per type), labels from a teacher net (other seed) + N(0, 0.01) noise
TRAIN_CONFIGS, TRAIN_NMIN, TRAIN_NMAX, TRAIN_DENSITY, TRAIN_STRAIN = 64, 32, 512, 0.07, 0.03
TRAIN_SEED = 303


def train_workload(dev, nconf=TRAIN_CONFIGS, seed=TRAIN_SEED):
    """The ragged training batch and its labels (teacher net of the same architecture)."""
    from matpl_gb300 import data, dp, params as P, structures
    rng = np.random.default_rng(seed)
    counts = rng.integers(TRAIN_NMIN, TRAIN_NMAX + 1, nconf)
    sts = [structures.random_packed(int(n), TRAIN_DENSITY, [72, 8], [1 / 3, 2 / 3],
                                    seed=seed + 1 + k, strain=TRAIN_STRAIN)
           for k, n in enumerate(counts)]
    cfg = P.DPConfig(atom_type=[72, 8], maxNeighborNum=100, Rmax=RC, Rmin=RMIN)
    batch = data.ragged_batch(cfg, sts, device=dev)
    ln, idr = batch["list_neigh"], batch["ImageDR"]
    davg, dstd = P.calc_stat(cfg, ln.cpu().numpy(), idr.cpu().numpy(),
                             batch["type_map"].cpu().numpy())
    teacher = dp.DP(cfg, P.init_params(cfg, SEED_W + 100), davg, dstd, precision="float64",
                    device=dev)
    present = teacher.present_types(cfg.atom_type)
    lab = teacher.evaluate(ln, batch["type_map"], present, idr, 0)
    g = torch.Generator(device=dev).manual_seed(5)
    E = data.config_energies(lab["Ei_atom"], batch["config_of_atom"], nconf)
    batch["Etot"] = (E + 0.01 * torch.randn(E.shape, generator=g, device=dev,
                                            dtype=torch.float64)).float()
    batch["Force"] = (lab["Force"] + 0.01 * torch.randn(lab["Force"].shape, generator=g,
                                                         device=dev, dtype=torch.float64)).float()
    batch["ImageDR"] = idr.float()
    return cfg, batch, davg, dstd, counts


def run_train(args, ws, local, steps, warmup, plain_steps):
    """Force-loss training step (E-MSE over the configurations + F-MSE, Adam) on the ragged
    batch of 64 uneven Hf:O configurations (one concatenated image, no per-composition
    clusters): the fused step (fused E/F, hand-written embedding double-backward, torch fitting
    part) against the plain step (env matrix + torch nets + second-order autograd through this
    library's force / virial ops, the reference's structure), both FP32."""
    from matpl_gb300 import _lib, params as P, train
    dev = torch.device("cuda", local)
    cfg, batch, davg, dstd, counts = train_workload(dev, args.train_configs)
    natoms = int(counts.sum())
    prm = P.init_params(cfg, SEED_W)

    def timed(step, n, w):
        for _ in range(w):
            step()
        torch.cuda.synchronize()
        barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            step()
        e1.record()
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / n, ws)

    # fused step, eager (per-kernel times from the library's events)
    emodel = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float32, device=dev)
    eopt = torch.optim.Adam(emodel.parameters(), lr=1e-4, fused=True)
    etrainer = train.FusedTrainer(emodel, "mixed")
    etrainer.step([batch], eopt)
    _lib.profile_begin(max(4096, steps * 32))
    eager_ms = timed(lambda: etrainer.step([batch], eopt), max(3, steps // 3), 1)
    prof = _lib.profile_collect()
    del etrainer, emodel, eopt
    # fused step captured in one CUDA graph (the headline of this workload): its E / F
    # evaluation on the tcgen05 tensor cores (BF16x3), the FP32-evaluation form beside it
    fmodel = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float32, device=dev)
    fopt = torch.optim.Adam(fmodel.parameters(), lr=1e-4, capturable=True, fused=True)
    graphed = train.GraphedTrainer(train.FusedTrainer(fmodel, "mixed"), fopt)
    fused_ms = timed(lambda: graphed.step(batch), steps, warmup)
    del graphed, fopt, fmodel
    smodel = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float32, device=dev)
    sopt = torch.optim.Adam(smodel.parameters(), lr=1e-4, capturable=True, fused=True)
    sgraphed = train.GraphedTrainer(train.FusedTrainer(smodel), sopt)
    simt_ms = timed(lambda: sgraphed.step(batch), steps, warmup)
    del sgraphed, sopt, smodel
    pmodel = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float32, device=dev)
    popt = torch.optim.Adam(pmodel.parameters(), lr=1e-4, fused=True)
    torch.cuda.reset_peak_memory_stats(dev)
    plain_ms = timed(lambda: train.train_step(pmodel, [batch], popt), plain_steps, 1)
    plain_peak = torch.cuda.max_memory_allocated(dev)
    # gradient agreement of the two paths at one parameter point
    m1 = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float32, device=dev)
    m2 = train.DPTrainModel(cfg, prm, davg, dstd, dtype=torch.float32, device=dev)
    train.FusedTrainer(m1, "mixed").loss_and_backward(batch)
    train.loss_fn(m2, batch)[0].backward()
    worst = 0.0
    for k in m1.names:
        a, b = m1.param(k).grad, m2.param(k).grad
        worst = max(worst, ((a - b).abs().max() / (b.abs().max() + 1e-30)).item())
    per_kernel = {k: {"ms_per_launch": v[0] / v[1], "launches": v[1]} for k, v in prof.items()}
    pairs = int((batch["list_neigh"] > 0).sum())
    # roofline of the dominant library kernel: the embedding double-backward recomputes the
    # forward and runs the reverse of the tangent pass, ~6.6 kflop per occupied pair
    roof = None
    if "dp_dual_bwd" in per_kernel:
        t = per_kernel["dp_dual_bwd"]["ms_per_launch"] * 1e-3
        ach = 6600.0 * pairs / t / 1e12
        simt_peak = sm_count() * 128 * 2 * 2070.0 * 1e6 / 1e12
        roof = {"kernel": "dp_dual_bwd", "bound": "simt fp32", "achieved": ach,
                "peak": simt_peak, "unit": "TFLOP/s", "frac": ach / simt_peak,
                "peak_source": "nominal FP32 SIMT at 2070 MHz",
                "algorithmic_flops_per_launch": 6600.0 * pairs}
    return {
        "metric": TRAIN_METRIC, "value": ws * natoms / (fused_ms * 1e-3), "unit": "atom-steps/s",
        "ms_per_step": fused_ms, "steps": steps, "warmup": warmup,
        "dtype": "f32 (E / F evaluation bf16x3 tensor, f32 accumulation)",
        "config": {"workload": f"DP se_e2_a force-loss training step (E-MSE + F-MSE, Adam) on a "
                               f"ragged batch of {TRAIN_CONFIGS} Hf:O configurations, atom counts "
                               f"U[{TRAIN_NMIN}, {TRAIN_NMAX}] ({natoms:,} atoms), "
                               f"{TRAIN_DENSITY} atoms/A^3, {TRAIN_STRAIN:.0%} cell strain, m=100/type, "
                               "teacher labels + N(0, 0.01)",
                   "natoms": natoms, "pairs": pairs, "configurations": TRAIN_CONFIGS,
                   "batching": "one concatenated image (data.ragged_batch), energies per "
                               "configuration",
                   "plain_fp32": {"form": "env matrix + torch nets + second-order autograd through "
                                          "this library's force / virial ops",
                                  "ms_per_step": plain_ms, "value": ws * natoms / (plain_ms * 1e-3),
                                  "steps": plain_steps, "peak_memory_bytes": plain_peak},
                   "fused_eager_ms_per_step": eager_ms,
                   "fused_fp32_evaluation_ms_per_step": simt_ms,
                   "capture": "whole fused step (evaluation, dual kernels, fitting part, backward, "
                              "Adam) in one CUDA graph, replayed per step",
                   "speedup_vs_plain_fp32": plain_ms / fused_ms,
                   "gradient_max_rel_diff_fused_vs_plain": worst},
        "kernels": per_kernel, "roofline": roof,
    }


NEP_TRAIN_METRIC = ("NEP force-loss training step atom-steps/s (E + F + virial loss, Adam; "
                    "hand-written descriptor second derivatives)")
NEP_TRAIN_NATOMS = 20_000
NEP_TRAIN_CPU_SAMPLE = 2000


def nep_train_setup(dev, natoms, seed=NEP_SEED_STRUCT + 7):
    """A NEP training batch: the NEP workload's model on a `natoms` box of the same density,
    split into four frames (num_atom), exact lists from calculate_neighbor, q_scaler from the
    box's descriptors, labels from a teacher NEP (other seed) plus N(0, 0.01) noise."""
    from matpl_gb300 import nep as NP, ops, structures
    cfg = NP.NepConfig(atom_type=list(NEP_ELEMENTS))
    per = max(1, natoms // 4)
    sts = [structures.random_packed(per, NEP_DENSITY, NEP_ELEMENTS, [0.25] * 4, seed=seed + k)
           for k in range(4)]
    fr = NP.frames_from_structures(sts, cfg.cutoff[0])
    c = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)  # noqa: E731
    na, tm = c(fr.num_atom.reshape(-1, 1), torch.int64), c(fr.type_map, torch.int64)
    bx, bo, nc = c(fr.box, torch.float64), c(fr.box_orig, torch.float64), c(fr.num_cell, torch.int64)
    pos = c(fr.position, torch.float64)
    at = torch.arange(cfg.ntypes, device=dev)
    cr, ca = ops.calculate_maxneigh(na, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1], cfg.ntypes,
                                    tm, False)
    lists = ops.calculate_neighbor(na, tm, at, bx, bo, nc, pos, cfg.cutoff[0], cfg.cutoff[1],
                                   int(cr.max()), int(ca.max()), True)
    prm = NP.init_params(cfg, NEP_SEED_W, energy_shift=-3.0)
    m64 = NP.NEP(cfg, prm, "float64", device=dev)
    feats = m64.descriptor(lists[0], lists[2], lists[4], lists[1], lists[3], lists[5], na, tm)
    qs = NP.calc_q_scaler(cfg, feats).cpu()
    prm["q_scaler"] = qs
    tprm = NP.init_params(cfg, NEP_SEED_W + 50, energy_shift=-3.0)
    tprm["q_scaler"] = qs
    lab = NP.NEP(cfg, tprm, "float64", device=dev).evaluate(lists[0], lists[2], lists[4],
                                                            lists[1], lists[3], lists[5], na, tm)
    g = torch.Generator(device=dev).manual_seed(3)
    labels = {"Etot": lab["Etot"].reshape(-1) + 0.01 * torch.randn(len(sts), generator=g,
                                                                   device=dev, dtype=torch.float64),
              "Force": lab["Force"].double() + 0.01 * torch.randn(lab["Force"].shape, generator=g,
                                                                  device=dev, dtype=torch.float64),
              "Virial": lab["Virial"].double()}
    return cfg, fr, prm, lists, na, tm, labels


def run_nep_train(args, ws, local, steps, warmup):
    """NEP force-loss training step on a 20,000-atom four-frame batch: NEPTrain (NEP.forward's
    CUDA branch on calculateNepFeat / calculateNepMbFeat with hand-written first and second
    backward, calculateNepForce / calculateNepVirial), loss = per-atom energy MSE + force MSE +
    virial MSE, loss.backward(), Adam; the FP32 step captured in one CUDA graph (timed), eager
    FP32 and FP64 beside it."""
    from matpl_gb300 import _lib, nep_ops
    from matpl_gb300.nep_train import GraphedNepTrainer, NEPTrain
    dev = torch.device("cuda", local)
    cfg, fr, prm, lists, na, tm, lab = nep_train_setup(dev, args.nep_train_atoms)
    N = fr.natoms
    na_h = torch.tensor(fr.num_atom.reshape(-1, 1))
    nep_ops.set_check_errors(False)

    def make(dt):
        model = NEPTrain(cfg, prm, dtype=dt, device=dev)
        opt = torch.optim.Adam(model.parameters(), lr=1e-4, fused=True)
        tr = GraphedNepTrainer(model, opt, w_e=1.0, w_f=1.0, w_v=1e-4)
        b = batch(dt)
        tidx = model.type_index(tm)

        def step():
            opt.zero_grad(set_to_none=True)
            loss = tr.loss(b, tidx)
            loss.backward()
            opt.step()
            return loss
        return step

    def batch(dt):
        return {"NN_r": lists[0], "NL_r": lists[2], "Ri_r": lists[4].to(dt), "NN_a": lists[1],
                "NL_a": lists[3], "Ri_a": lists[5].to(dt), "type_map": tm, "num_atom": na_h,
                "per_atom": torch.tensor(fr.num_atom, dtype=dt, device=dev),
                "Etot": lab["Etot"].to(dt), "Force": lab["Force"].to(dt),
                "Virial": lab["Virial"].to(dt)}

    def timed(step, n, w):
        for _ in range(w):
            step()
        torch.cuda.synchronize()
        barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            loss = step()
        e1.record()
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / n, ws), float(loss.detach())

    # graphed FP32 step (the headline of this workload)
    gmodel = NEPTrain(cfg, prm, dtype=torch.float32, device=dev)
    gopt = torch.optim.Adam(gmodel.parameters(), lr=1e-4, capturable=True, fused=True)
    graphed = GraphedNepTrainer(gmodel, gopt, w_e=1.0, w_f=1.0, w_v=1e-4)
    b32 = batch(torch.float32)
    gms, gloss = timed(lambda: graphed.step(b32), steps, warmup)
    graphed.check_errors()
    del graphed, gmodel, gopt
    # eager FP32 with per-kernel times, eager FP64
    s32 = make(torch.float32)
    for _ in range(warmup):
        s32()
    _lib.profile_begin(max(4096, steps * 64))
    ms32, loss32 = timed(s32, steps, 0)
    prof = _lib.profile_collect()
    s64 = make(torch.float64)
    ms64, loss64 = timed(s64, max(3, steps // 2), 2)
    nep_ops.check_errors(dev)
    nep_ops.set_check_errors(True)
    per_kernel = {k: {"ms_per_step": v[0] / steps, "launches_per_step": v[1] / steps}
                  for k, v in prof.items()}
    return {"metric": NEP_TRAIN_METRIC, "value": ws * N / (gms * 1e-3), "unit": "atom-steps/s",
            "ms_per_step": gms, "steps": steps, "warmup": warmup, "dtype": "f32",
            "config": {"workload": f"NEP training batch of 4 frames, {N:,} atoms, four elements, "
                                   f"{NEP_DENSITY} atoms/A^3, rc 6 / 4 A, n_max 4 / 4, basis 8 / 8, "
                                   "l_max 4 / 2 / 1, 30 hidden; teacher labels (E, F, V)",
                       "natoms": N, "loss_graphed_fp32": gloss,
                       "capture": "whole step (forward, create_graph forces, loss, backward through "
                                  "the hand-written second derivatives, Adam) in one CUDA graph",
                       "eager_fp32": {"ms_per_step": ms32, "value": ws * N / (ms32 * 1e-3),
                                      "loss": loss32},
                       "eager_fp64": {"ms_per_step": ms64, "value": ws * N / (ms64 * 1e-3),
                                      "loss": loss64},
                       "form": "autograd over this library's operators in the reference's op "
                               "structure; the force path takes the descriptor's d12 gradient "
                               "alone, forces and virial in one kernel reading the (r, x, y, z) "
                               "rows, all elements' fitting nets in one product"},
            "kernels": per_kernel}


def cpu_baseline_nep_train(steps=5):
    """The reference's NEP training gradient on the host cores: the oracle port of the CPU
    branch of NEP.forward with second-order autograd (torch FP64, all host threads) on a
    bounded 2,000-atom sample of the same model and density."""
    from oracle import nep_oracle as NO
    from matpl_gb300 import nep as NP, structures
    ncores = os.cpu_count() or 1
    torch.set_num_threads(ncores)
    cfg = NP.NepConfig(atom_type=list(NEP_ELEMENTS))
    st = structures.random_packed(NEP_TRAIN_CPU_SAMPLE, NEP_DENSITY, NEP_ELEMENTS, [0.25] * 4,
                                  seed=NEP_SEED_STRUCT + 9)
    fr = NP.frames_from_structures([st], cfg.cutoff[0])
    cr, ca = NO.maxneigh(fr, cfg.cutoff[0], cfg.cutoff[1])
    L = NO.neighbor(fr, cfg.cutoff[0], cfg.cutoff[1], int(cr.max()), int(ca.max()))
    prm = NP.init_params(cfg, NEP_SEED_W, energy_shift=-3.0)
    rng = np.random.default_rng(1)
    N = fr.natoms
    gE, gF, gV = rng.standard_normal(1), rng.standard_normal((N, 3)), rng.standard_normal((1, 9))
    ts = []
    for _ in range(steps + 1):
        t0 = time.perf_counter()
        NO.train_grads(cfg, prm, fr.num_atom, fr.type_map, L[2], L[4], L[3], L[5], gE, gF, gV)
        ts.append(time.perf_counter() - t0)
    med = statistics.median(ts[1:])
    return {"value": N / med, "unit": "atom-steps/s", "cores": ncores, "kind": "port",
            "sample": f"{N}-atom four-element box, FP64, training gradient of an E + F + V loss "
                      f"(second-order autograd through the CPU descriptor), median of {steps}",
            "sec_per_step": med}


def run_nep_train_line(args, ws, rank, local):
    torch.cuda.set_device(local)
    from matpl_gb300 import _lib
    _lib.load()
    steps = args.steps if args.steps_given else 20
    r = run_nep_train(args, ws, local, steps=steps, warmup=args.warmup)
    if rank == 0 and not args.no_cpu_baseline:
        r["cpu_baseline"] = cpu_baseline_nep_train()
    if rank != 0:
        return
    line = {"metric": r.pop("metric"), "value": r.pop("value"), "unit": r.pop("unit"),
            "n_gpus": ws, "steps": r.pop("steps"), "warmup": r.pop("warmup"),
            "ms_per_step": r.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": r.pop("dtype"), "data": "synthetic", **r}
    print(json.dumps(line))


VARIANT_ATOMS = 8000


def calcops_reference_gpu(ln, dev, reps=10):
    """CalcOps_cuda calculateForce / calculateVirial: the reference's own kernels
    (src/op/kernel/calculateForce.cu, calculateVirial.cu, built unmodified for sm_103a from a
    staged copy, baseline/ref_gpu.py) against this library's operators on the headline list
    (32,000 atoms, S = 300 slots), FP64, the same seeded dE / Ri_d / Rij / centre term.  Each op
    is timed as the torch op runs it: the reference's output set-up (CalcOps.cpp:17-20,
    :181-184: zero-fill, centre-term copy) + its launcher, against the C-ABI call."""
    try:
        from baseline import ref_gpu
    except ImportError as e:
        return {"unavailable": f"comparator module not importable: {e}"}
    from matpl_gb300 import _lib
    from matpl_gb300._lib import check, ptr
    rl = ref_gpu.load()
    if rl is None:
        return {"unavailable": "comparator library not built (reference GPU sources not staged)"}
    lib = _lib.load()
    B, N, S = ln.shape
    nb = (ln.to(torch.int32) - 1).contiguous()          # 0-based, -1 = empty slot
    g = torch.Generator(device=dev).manual_seed(5)
    f64 = dict(dtype=torch.float64, device=dev)
    dE = torch.randn(B, N, 4 * S, generator=g, **f64)
    Ri_d = torch.randn(B, N, 4 * S, 3, generator=g, **f64)
    Rij = torch.randn(B, N, S, 3, generator=g, **f64)
    Fc = torch.randn(B, N, 3, generator=g, **f64)
    fo, fr = torch.empty(B, N, 3, **f64), torch.empty(B, N, 3, **f64)
    vo, vr = torch.empty(B, 9, **f64), torch.empty(B, 9, **f64)
    avo, avr = torch.empty(B, N, 9, **f64), torch.empty(B, N, 9, **f64)
    st = torch.cuda.current_stream(dev).cuda_stream
    di = dev.index if dev.index is not None else torch.cuda.current_device()

    def ours_f():
        check(lib.matpl_calc_force(_lib.MATPL_F64, ptr(nb), ptr(dE), ptr(Ri_d), ptr(Fc), B, N,
                                   S, 0, ptr(fo), st), "matpl_calc_force")

    def ref_f():
        fr.zero_()
        fr.copy_(Fc)
        rl.refcalc_force(0, ptr(nb), ptr(dE), ptr(Ri_d), B, N, S, ptr(fr), 0, di)

    def ours_v():
        check(lib.matpl_calc_virial(_lib.MATPL_F64, ptr(nb), ptr(dE), ptr(Rij), ptr(Ri_d), B, N,
                                    S, 0, ptr(vo), ptr(avo), st), "matpl_calc_virial")

    def ref_v():
        vr.zero_()
        avr.zero_()
        rl.refcalc_virial(0, ptr(nb), ptr(dE), ptr(Rij), ptr(Ri_d), B, N, S, ptr(vr), ptr(avr),
                          0, di)

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    rel = lambda a, b: float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))  # noqa: E731
    out = {"config": f"FP64, batch {B}, {N} atoms, {S} slots, "
                     f"{int((nb >= 0).sum())} occupied; inputs {(dE.numel() + Ri_d.numel() + Rij.numel()) * 8 / 1e9:.2f} GB"}
    for name, o, r, res in (("calculateForce", ours_f, ref_f, lambda: [(fo, fr)]),
                            ("calculateVirial", ours_v, ref_v, lambda: [(vo, vr), (avo, avr)])):
        o(); r()
        torch.cuda.synchronize()
        err = max(rel(a, b) for a, b in res())
        t_o, t_r = timed(o), timed(r)
        out[name] = {"ours_ms": t_o, "reference_ms": t_r, "speedup": t_r / t_o,
                     "max_rel_diff": err}
    return out


def run_dp_variants(args, ws, local):
    """The DP model variants evaluated through this library's operators in the reference's own
    structure (environment matrix, per type-pair contraction, fitting nets, autograd dE/dRi,
    calculateForce / calculateVirial): the compressed model (order-5 table through
    calculateCompress) and the type-embedding model, FP32, on an 8,000-atom box of the
    headline's density; E + F + V per step, CUDA events."""
    from matpl_gb300 import compress as C, ops, params as P
    from matpl_gb300.typedp import TypeDP, init_type_params, fused_model as typedp_fused
    dev = torch.device("cuda", local)
    st, cfg, prm = make_workload(VARIANT_ATOMS)
    tm = torch.tensor(st.types, dtype=torch.int32, device=dev)
    ln, idr = ops.find_neighbore(tm, torch.tensor(st.frac, device=dev),
                                 torch.tensor(st.lattice, device=dev), 2, M_NEIGH, RC, RC)
    davg, dstd = P.calc_stat(cfg, ln.cpu().numpy(), idr.cpu().numpy(), st.types)
    idr32 = idr.float()
    r = idr[..., 0][ln > 0]
    u = (r - RMIN) / (RC - RMIN)
    vv = torch.where(r < RMIN, torch.ones_like(r),
                     torch.where(r < RC, u ** 3 * (-6 * u * u + 15 * u - 10) + 1, torch.zeros_like(r)))
    sij_max = float((vv / r).max())
    out = {}

    def timed(model, n=5):
        for _ in range(2):
            model(ln, tm, cfg.atom_type, idr32, 0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            model(ln, tm, cfg.atom_type, idr32, 0)
        e1.record()
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / n, ws)

    comp = C.build_table(cfg, prm, davg, dstd, sij_max, 0.01, 5, device=dev)
    ms = timed(C.CompressedDP(cfg, prm, davg, dstd, comp, dtype=torch.float32, device=dev))
    out["compressed_order5"] = {"ms_per_step": ms, "value": ws * VARIANT_ATOMS / (ms * 1e-3),
                                "table_rows": int(comp["table"].shape[1])}
    # the same table in the fused kernels (matpl_dp_eval with ctable): FP32, and the mixed
    # form (table on SIMT, fitting nets on the tensor cores)
    for prec in ("float32", "mixed"):
        fused = C.fused_model(cfg, prm, davg, dstd, comp, prec, dev)
        fused.check_errors = False
        ms = timed(fused)
        out[f"compressed_order5_fused_{prec}"] = {"ms_per_step": ms,
                                                  "value": ws * VARIANT_ATOMS / (ms * 1e-3)}
    vec = {3: [0.0185, 0.0216, 0.3], 14: [0.1204, 0.0985, 0.2]}
    tprm = init_type_params(cfg, 3, SEED_W)
    ms = timed(TypeDP(cfg, tprm, davg, dstd, vec, dtype=torch.float32, device=dev))
    out["type_embedding"] = {"ms_per_step": ms, "value": ws * VARIANT_ATOMS / (ms * 1e-3)}
    # the same model folded into per-pair nets in the fused kernels (FP32 and BF16x3 tcgen05)
    for prec in ("float32", "mixed"):
        fm = typedp_fused(cfg, tprm, davg, dstd, vec, precision=prec, device=dev)
        fm.check_errors = False
        ms = timed(fm)
        out[f"type_embedding_fused_{prec}"] = {"ms_per_step": ms,
                                               "value": ws * VARIANT_ATOMS / (ms * 1e-3)}
    return {"metric": "DP variant E+F+virial atom-steps/s (reference structure on this "
                      "library's operators, FP32; both also in the fused kernels)",
            "unit": "atom-steps/s",
            "config": {"workload": f"{VARIANT_ATOMS}-atom Li/Si box, m=150/type, Rc 6",
                       "cpu_baseline": "none: the reference path of these variants is its "
                                       "Python model, which the bench does not run; parity "
                                       "is pinned by the golden fixtures"},
            **out}


DATA_METRIC = "dataset statistics pass (neighbor search + davg/dstd sums) images/s"
DATA_IMAGES = 2048


def run_data(args, ws, local):
    """The data path's statistics pass over a dataset of 2,048 Li/Si images (108 atoms, the
    headline density and model, m = 150): neighbor lists of every image and the per-type sums
    behind davg / dstd (matpl_gb300.data.image_stats), images of one shape batched into one
    launch; host wall clock.  CPU baseline: the oracle port (C NeighConst restatement + the
    numpy restatement of calc_stat's sums) on a 64-image sample."""
    from matpl_gb300 import data as D, params as P, structures
    from oracle import neigh
    cfg = P.DPConfig(atom_type=list(ELEMENTS), maxNeighborNum=M_NEIGH, Rmax=RC, Rmin=RMIN)
    base = [structures.random_packed(108, DENSITY, ELEMENTS, [0.5, 0.5], seed=900 + k)
            for k in range(16)]
    ims = []
    for k in range(DATA_IMAGES):       # 16 compositions, jittered positions
        b = base[k % 16]
        rng = np.random.default_rng(k)
        ims.append(structures.Structure(b.lattice, np.mod(b.frac + 0.002 * rng.standard_normal(
            b.frac.shape), 1.0), b.types, b.elements))
    D.image_stats(cfg, ims[:32])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    D.image_stats(cfg, ims)
    torch.cuda.synchronize()
    sec = max_over_ranks(time.perf_counter() - t0, ws)
    cb = None
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        for st in ims[:64]:
            tm = D.model_types(st, cfg.atom_type)
            ln, idr = neigh.find_neighbore(tm, st.frac, st.lattice, cfg.ntypes, M_NEIGH, RC,
                                           [RC, RC])
            neigh.env_sums(cfg, ln, idr, tm)
        ct = time.perf_counter() - t0
        cb = {"value": 64 / ct, "unit": "images/s", "cores": 1, "kind": "port",
              "sample": "64 of the same images, C restatement of NeighConst + numpy sums"}
    return {"metric": DATA_METRIC, "value": ws * DATA_IMAGES / sec, "unit": "images/s",
            "seconds": sec, "config": {"workload": f"{DATA_IMAGES} Li/Si images of 108 atoms "
                                                   "(16 compositions), m = 150, Rc 6",
                                       "timing": "host wall clock, one pass"},
            "cpu_baseline": cb}


MD_METRIC = ("batched replica MD atom-steps/s (velocity Verlet, DP mixed, all replicas in one "
             "ragged step, 10 steps per CUDA-graph launch, Verlet skin 1.0 A)")
MD_REPLICAS, MD_NMIN, MD_NMAX, MD_SEED = 256, 64, 2048, 77
MD_STEPS_PER_GRAPH = 10


def md_replicas(n=MD_REPLICAS, seed=MD_SEED):
    """Cu FCC replicas (a = 3.615 A, sigma = 0.05 A) with atom counts log-uniform in
    [64, 2048]: the count picks nx = ny = round((N/4)^(1/3)) and nz = round(N / (4 nx ny))
    conventional cells, so the counts are 4 nx ny nz (uneven)."""
    from matpl_gb300 import structures
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n):
        N = float(np.exp(rng.uniform(np.log(MD_NMIN), np.log(MD_NMAX))))
        nc = N / 4.0
        nx = max(2, int(round(nc ** (1.0 / 3.0))))
        nz = max(2, int(round(nc / (nx * nx))))
        out.append(structures.fcc(3.615, (nx, nx, nz), 0.05, seed=seed + r))
    return out


def run_md(args, ws, local, steps):
    """256 Cu replicas of uneven size, DP (1 type, m = 100, Rc 6, random weights N(0, 1/fan_in)),
    Maxwell-Boltzmann velocities at 300 K, dt = 1 fs: `steps` velocity-Verlet steps of every
    replica.  All replicas form one ragged atom array: per step one drift (+ rebuild flag), the
    gated skin-list build (Rc + 1 A, run only after some atom moved > 0.5 A), one cutoff filter,
    one mixed-form evaluation, one kick; 10 steps per CUDA-graph launch.  The evaluation's tile
    shape is autotuned on the replicas' own list.  Reports the total-energy drift per atom (FP64
    energy sums) and the number of list builds."""
    from matpl_gb300 import autotune, md, params as P, structures
    dev = torch.device("cuda", local)
    autotune.set_tuning(0, 0)              # the headline's tuned tile shape is for its own box
    cfg = P.DPConfig(atom_type=[29], maxNeighborNum=100, Rmax=6.0, Rmin=0.5)
    reps = md_replicas()
    st = structures.fcc(3.615, (4, 4, 4), 0.05, seed=1)
    from matpl_gb300 import ops
    l0, r0 = ops.find_neighbore(torch.tensor(st.types, device=dev), torch.tensor(st.frac, device=dev),
                                torch.tensor(st.lattice, device=dev), 1, 100, 6.0, 6.0)
    davg, dstd = P.calc_stat(cfg, l0.cpu().numpy(), r0.cpu().numpy(), st.types)
    prm = P.init_params(cfg, SEED_W)
    sim = md.ReplicaMD(cfg, prm, davg, dstd, reps, [63.546], dt_fs=1.0, precision="mixed",
                       device=dev, skin=1.0, steps_per_graph=MD_STEPS_PER_GRAPH)
    tuning = "automatic"
    if not args.no_tune:
        t = autotune.tune_dp_mixed(sim.model, sim.ln, sim.types, sim.present, sim.idr,
                                   num_neigh=sim.nn)
        tuning = {"group_atoms": t["group_atoms"], "ctas_per_sm": t["ctas_per_sm"]}
    sim.capture()
    e0 = sim.energies().sum(1)
    n = sim.natoms()
    b0 = sim.rebuilds()
    torch.cuda.synchronize()
    barrier(ws)
    e_0, e_1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_0.record()
    chunk = max(MD_STEPS_PER_GRAPH, (steps // 10) // MD_STEPS_PER_GRAPH * MD_STEPS_PER_GRAPH)
    worst = 0.0
    done = 0
    while done < steps:
        k = min(chunk, steps - done)
        sim.step(k)
        done += k
        e = sim.energies().sum(1)           # one sync per chunk
        worst = max(worst, float(np.max(np.abs(e - e0) / n)))
    e_1.record()
    torch.cuda.synchronize()
    sim.check_errors()
    autotune.set_tuning(0, 0)
    ms = max_over_ranks(e_0.elapsed_time(e_1) / steps, ws)
    drift = (e - e0) / n
    pairs = int(sim.nn.sum())
    return {"metric": MD_METRIC, "value": ws * sim.natoms_total / (ms * 1e-3),
            "unit": "atom-steps/s", "ms_per_step": ms, "steps": steps,
            "config": {"workload": f"{len(reps)} Cu FCC replicas, atom counts log-uniform in "
                                   f"[{MD_NMIN}, {MD_NMAX}] ({int(n.min())}..{int(n.max())}, "
                                   f"{sim.natoms_total} atoms), DP m=100 Rc 6, 300 K, dt 1 fs, "
                                   "Verlet skin 1.0 A (rebuild when an atom moved > 0.5 A)",
                       "natoms_total": sim.natoms_total, "pairs_within_rc": pairs,
                       "steps_per_graph_launch": MD_STEPS_PER_GRAPH,
                       "list_builds_in_timed_steps": sim.rebuilds() - b0,
                       "skin_list_capacity_per_type": sim.cap,
                       "energy_drift_per_atom_eV": {"final_mean_abs": float(np.mean(np.abs(drift))),
                                                    "max_abs_over_run": worst},
                       "tile_tuning": tuning}}


LMP_METRIC = ("LAMMPS pair_style DP step atom-steps/s (LAMMPS host positions + full list in, "
              "host forces / energy / virial out)")
LMP_SKIN = 1.0      # neighbor 1.0 bin (the reference's LAMMPS demo)


def lammps_bytes(inum, nall, entries, S, es):
    """Unique bytes the slot conversion must move: the list (4 B per entry), ilist + jstart,
    positions and types of every atom once, and the slot arrays it writes (list_neigh 4 B +
    ImageDR 4 * es B per slot) + type_map."""
    return 4 * entries + inum * (4 + 8) + nall * (24 + 4) + inum * S * (4 + 4 * es) + 4 * inum


def cpu_baseline_lammps(s, cfg, t2m, sample):
    """The reference's host-side per-step stage, generate_neighdata (oracle restatement in C,
    one core, like the reference's loop), on the first `sample` list rows of the same system
    (all of them by default); median of up to 20 runs within about 10 s."""
    from oracle import lammps as OL
    n = min(sample, s["nlocal"])
    js = s["jstart"][:n + 1]
    jf = s["jflat"][:js[-1]]
    reps = []
    t_end = time.perf_counter() + 10.0
    while time.perf_counter() < t_end and len(reps) < 20:
        t0 = time.perf_counter()
        OL.neighdata(s["ilist"][:n], js, jf, s["x"], s["type"], t2m, cfg.ntypes,
                     cfg.maxNeighborNum, cfg.Rmax)
        reps.append(time.perf_counter() - t0)
    t = statistics.median(reps)
    return {"value": n / t, "unit": "atom-steps/s", "cores": 1, "kind": "port",
            "sample": f"generate_neighdata (pair_matpl.cpp:522-616) restated in C, {n} list rows "
                      f"of the same system, median of {len(reps)} runs; the reference then copies "
                      "the slot arrays to the GPU and runs its TorchScript model, not timed here"}


def run_lammps(args, ws, local, steps, warmup):
    """The headline system as LAMMPS hands it to a full-list pair style: 32,000 local atoms,
    periodic images within Rc + skin (7 A) as ghost atoms, a full list per local atom in random
    order (a neighbor-bin build), pair_coeff * * 3 14.  One step = PairMATPL.compute on the
    host arrays: pack + one host-to-device copy, slot conversion on the GPU, fused E/F/V with
    ghost rows, one device-to-host copy of forces (local + ghost), energy, virial."""
    from matpl_gb300 import _lib, dp, lammps as L, ops, params as P
    dev = torch.device("cuda", local)
    st, cfg, prm = make_workload(args.lammps_atoms)
    l0, r0 = ops.find_neighbore(torch.tensor(st.types), torch.tensor(st.frac, device=dev),
                                torch.tensor(st.lattice), cfg.ntypes, cfg.maxNeighborNum, RC, RC)
    davg, dstd = P.calc_stat(cfg, l0.cpu().numpy(), r0.cpu().numpy(), st.types)
    s = L.lammps_system(st.lattice, st.cart, st.types + 1, RC + LMP_SKIN, seed=SEED_STRUCT)
    prec = args.precision
    model = dp.DP(cfg, prm, torch.as_tensor(davg), torch.as_tensor(dstd), precision=prec,
                  device=dev, check_errors=False)
    tuning = "automatic"
    if prec.startswith("mixed") and not args.no_tune:
        # tile shape of the mixed kernels, timed on this machine's own slot occupancy
        from matpl_gb300 import autotune
        tm0 = torch.tensor(st.types, dtype=torch.int32, device=dev)
        t = autotune.tune_dp_mixed(model, l0, tm0, [0, 1], r0.to(model.dtype))
        tuning = {"group_atoms": t["group_atoms"], "ctas_per_sm": t["ctas_per_sm"]}
    del l0, r0
    pair = L.PairMATPL(model, ELEMENTS, eatom_grouped=True, host_access=args.lammps_access)
    fn = L.firstneigh_of(s)
    nall = s["nlocal"] + s["nghost"]
    f = np.zeros((nall, 3))

    def step(p=pair):
        return p.compute(s["x"], s["type"], s["nlocal"], s["nghost"], s["ilist"],
                         s["numneigh"], fn, f_out=f)

    def wall(p, n, w):
        for _ in range(w):
            step(p)
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(n):
            r = step(p)
        return max_over_ranks((time.perf_counter() - t0) * 1e3 / n, ws), r

    wall_ms, r = wall(pair, steps, warmup)
    f_direct = r["f"].copy()
    staged = None
    if pair.host_access == "direct":
        sp = L.PairMATPL(model, ELEMENTS, eatom_grouped=True, host_access="staged")
        s_ms, s_r = wall(sp, max(5, steps // 2), 3)
        staged = {"ms_per_step": s_ms, "value": ws * s["nlocal"] / (s_ms * 1e-3),
                  "max_abs_force_diff_vs_direct": float(np.abs(s_r["f"] - f_direct).max())}
        sp.close()
        step()   # leave f from the in-place form
    # the same steps again with per-kernel CUDA events (device-time split)
    psteps = max(3, min(steps, 20))
    _lib.profile_begin(max(4096, psteps * 16))
    for _ in range(psteps):
        step()
    prof = _lib.profile_collect()
    S = cfg.ntypes * cfg.maxNeighborNum
    es = 8 if prec == "float64" else 4
    entries = int(s["jflat"].size)
    nbytes = lammps_bytes(s["nlocal"], nall, entries, S, es)
    peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(HERE, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    nb_ms, nb_n = prof.get("lmp_neighbors", (0.0, 1))
    nb_avg = nb_ms / max(nb_n, 1)
    achieved = nbytes / (nb_avg * 1e-3) / 1e9 if nb_avg > 0 else None
    if pair.host_access == "direct":
        # copies: x, type, ilist, numneigh in; the lists are read in place over NVLink-C2C
        # and the results written in place (host bytes the GPU reads / writes per step)
        h2d = nall * 28 + s["nlocal"] * 8 + 4 * entries + 8 * s["nlocal"]
        d2h = 8 * (3 * nall + s["nlocal"] + 9)
    else:
        h2d = nall * 28 + s["nlocal"] * 12 + 8 + 4 * entries
        d2h = 8 * (3 * nall + s["nlocal"] + 9)
    ref_h2d = s["nlocal"] * (S * (4 + 32) + 4)   # int32 list + f64 dR + imagetype_map
    kernels = {k: {"ms_per_step": v[0] / psteps, "launches_per_step": v[1] / psteps}
               for k, v in prof.items()}
    tp = os.path.join(HERE, "profiles", "traffic.json")
    traffic = None
    if os.path.exists(tp):
        tr = json.load(open(tp)).get(f"lmp_neighbors:{'float64' if prec == 'float64' else 'mixed'}")
        traffic = tr["bytes_per_launch"] if tr else None
    return {"metric": LMP_METRIC, "value": ws * s["nlocal"] / (wall_ms * 1e-3),
            "unit": "atom-steps/s", "ms_per_step": wall_ms, "steps": steps, "warmup": warmup,
            "dtype": {"float32": "f32", "float64": "f64"}.get(prec, "bf16x3 tensor / f32 / f64 sums"),
            "config": {"workload": f"{s['nlocal']} local Li/Si atoms (the headline box) + "
                                   f"{s['nghost']} ghost atoms, full list within Rc + {LMP_SKIN} A "
                                   f"in random order ({entries} entries), pair_coeff * * 3 14",
                       "precision_form": prec, "nlocal": s["nlocal"], "nghost": s["nghost"],
                       "list_entries": entries, "host_access": pair.host_access,
                       "tile_tuning": tuning,
                       "staged_host_access": staged,
                       "timing": "host wall clock around PairMATPL.compute (it returns with the "
                                 "results on the host), max over ranks",
                       "reference_h2d_bytes_per_step": ref_h2d},
            "e2e": {"value": ws * s["nlocal"] / (wall_ms * 1e-3), "unit": "atom-steps/s",
                    "ms_per_step": wall_ms, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "kernels": kernels,
            "gpu_launches": int(sum(v[1] for v in prof.values()) / psteps * steps),
            "roofline": {"kernel": "lmp_neighbors", "bound": "hbm", "achieved": achieved,
                         "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak if achieved else None,
                         "algorithmic_bytes_per_launch": nbytes, "traffic": traffic,
                         "ms_per_launch": nb_avg,
                         "peak_source": "of measured (MEASURED_PEAKS.json)" if peaks
                         else "of fallback"},
            "energy": r["eng"]}, s, cfg


def run_lammps_line(args, ws, rank, local):
    torch.cuda.set_device(local)
    from matpl_gb300 import _lib
    _lib.load()
    steps = args.steps if args.steps_given else 50
    r, s, cfg = run_lammps(args, ws, local, steps=steps, warmup=args.warmup)
    if rank == 0 and not args.no_cpu_baseline:
        r["cpu_baseline"] = cpu_baseline_lammps(s, cfg, [0, 1], NATOMS)
    if rank != 0:
        return
    line = {"metric": r.pop("metric"), "value": r.pop("value"), "unit": r.pop("unit"),
            "n_gpus": ws, "steps": r.pop("steps"), "warmup": r.pop("warmup"),
            "ms_per_step": r.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": r.pop("dtype"), "data": "synthetic", **r}
    print(json.dumps(line))


def run_reference(args, ws, rank):
    if rank != 0:
        return
    # the requested K and W, bounded so that the host run stays within a few minutes
    steps = max(3, min(args.steps, 50))
    warm = max(3, min(args.warmup, 10))
    if args.workload == "nep":
        cb = cpu_baseline_nep(steps, warm)
        line = {"metric": NEP_METRIC, "value": cb["value"], "unit": "atom-steps/s",
                "n_gpus": args.gpus, "steps": steps, "warmup": warm,
                "ms_per_step": cb["sec_per_step"] * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": f"NEP, {NEP_CPU_SAMPLE}-atom sample of the 100,000-atom "
                                       "four-element 0.06/A^3 box", "device": "host CPU"},
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    cb = cpu_baseline_run(steps, warm)
    line = {"metric": METRIC, "value": cb["value"], "unit": "atom-steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": cb["sec_per_step"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"DP se_e2_a Li/Si, {CPU_SAMPLE}-atom sample of the 32k-atom "
                                   "0.05/A^3 box, m=150/type", "device": "host CPU"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "nep": None if args.no_nep else cpu_baseline_nep(3, 3)}
    print(json.dumps(line))


def run_ours(args, ws, rank, local):
    from matpl_gb300 import _lib, dp, ops, params as P
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    _lib.load()
    st, cfg, prm = make_workload()
    prec = args.precision
    types_d = torch.tensor(st.types, device=dev)
    frac_d = torch.tensor(st.frac, device=dev)
    lat_d = torch.tensor(st.lattice, device=dev)
    ln, idr = ops.find_neighbore(types_d, frac_d, lat_d, 2, M_NEIGH, RC, RC)   # overflow checked
    n_pairs = int((ln > 0).sum())
    sub = slice(0, 4000)
    davg, dstd = P.calc_stat(cfg, ln[:, sub].cpu().numpy(), idr[:, sub].cpu().numpy(), st.types[sub])
    m64 = dp.DP(cfg, prm, davg, dstd, precision="float64", device=dev)
    present = m64.present_types(cfg.atom_type)
    tm32 = types_d.to(torch.int32)
    r64 = m64.evaluate(ln, tm32, present, idr, 0)
    torch.cuda.synchronize()

    def make_step(form):
        model = dp.DP(cfg, prm, davg, dstd, precision=form, device=dev, check_errors=False)
        out_dt = model.dtype

        def step(frac, lat):
            # the fused step's lists: occupied slots + block lengths (no zero fill)
            l, r, c = ops.find_neighbore(types_d, frac, lat, 2, M_NEIGH, RC, RC,
                                         out_dtype=out_dt, check_overflow=False,
                                         occupied_only=True)
            return model.evaluate(l, tm32, present, r, 0, num_neigh=c)
        return model, step

    def accuracy(model, step):
        rr = step(frac_d, lat_d)
        torch.cuda.synchronize()
        if int(model.err.item()) != 0:
            raise RuntimeError(f"kernel error word {int(model.err.item())}")
        return {"force_rmse_vs_f64_eV_per_A": (rr["Force"].double() - r64["Force"]).pow(2).mean().sqrt().item(),
                "energy_err_per_atom_eV": abs(rr["Etot"].item() - r64["Etot"].item()) / NATOMS,
                "virial_max_abs_err_eV": (rr["Virial"] - r64["Virial"]).abs().max().item()}

    def timed(step, steps, warmup, sample_clocks):
        for _ in range(warmup):
            step(frac_d, lat_d)
        sampler = ClockSampler(local) if sample_clocks else None
        if sampler:
            sampler.start()
            time.sleep(0.3)
        torch.cuda.synchronize()
        barrier(ws)
        torch.cuda.synchronize()
        _lib.profile_begin(max(4096, steps * 16))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            step(frac_d, lat_d)
        e1.record()
        torch.cuda.synchronize()
        prof = _lib.profile_collect()
        barrier(ws)
        clocks = sampler.stop() if sampler else None
        ms = max_over_ranks(e0.elapsed_time(e1) / steps, ws)
        return ms, prof, clocks

    model, step = make_step(prec)
    tuning = None
    if prec.startswith("mixed") and not args.no_tune:
        from matpl_gb300 import autotune
        l0, r0, c0 = ops.find_neighbore(types_d, frac_d, lat_d, 2, M_NEIGH, RC, RC,
                                        out_dtype=model.dtype, occupied_only=True)
        tuning = autotune.tune_dp_mixed(model, l0, tm32, present, r0, num_neigh=c0)
        tuning["table"] = [(t["group_atoms"], t["ctas_per_sm"], round(t["ms"], 4))
                           for t in tuning["table"]]
        del l0, r0, c0
    acc = accuracy(model, step)
    ms, prof, clocks = timed(step, args.steps, args.warmup, True)
    value = replica_value(NATOMS, ms, ws)
    model_ms = sum(v[0] for k, v in prof.items() if not k.startswith("nb_")) / args.steps

    plain = None
    if prec != "float32" and not args.no_plain:
        pmodel, pstep = make_step("float32")
        pacc = accuracy(pmodel, pstep)
        psteps = max(10, args.steps // 3)
        pms, pprof, _ = timed(pstep, psteps, args.warmup, False)
        pmodel_ms = sum(v[0] for k, v in pprof.items() if not k.startswith("nb_")) / psteps
        plain = {"form": "float32 (plain SIMT)", "value": ws * NATOMS / (pms * 1e-3),
                 "ms_per_step": pms, "model_only_ms_per_step": pmodel_ms,
                 "model_only_value": ws * NATOMS / (pmodel_ms * 1e-3), **pacc}
        del pmodel
    plain64 = None
    if prec != "float64" and not args.no_plain:
        # the FP64 form: the arithmetic of the CPU arm, so the two compare like for like
        dmodel, dstep = make_step("float64")
        dsteps = 5
        dms, dprof, _ = timed(dstep, dsteps, 3, False)
        dmodel_ms = sum(v[0] for k, v in dprof.items() if not k.startswith("nb_")) / dsteps
        plain64 = {"form": "float64 (plain SIMT, the precision of the CPU baseline)",
                   "value": ws * NATOMS / (dms * 1e-3), "ms_per_step": dms,
                   "model_only_ms_per_step": dmodel_ms,
                   "model_only_value": ws * NATOMS / (dmodel_ms * 1e-3)}
        del dmodel

    # ---- end to end through host buffers
    out_dt = model.dtype
    frac_h = torch.tensor(st.frac).pin_memory()
    lat_h = torch.tensor(st.lattice).pin_memory()
    F_h = torch.empty(1, NATOMS, 3, dtype=out_dt).pin_memory()
    E_h = torch.empty(1, dtype=torch.float64).pin_memory()
    V_h = torch.empty(1, 9, dtype=torch.float64).pin_memory()

    def e2e_step():
        f = frac_h.to(dev, non_blocking=True)
        l = lat_h.to(dev, non_blocking=True)
        r = step(f, l)
        F_h.copy_(r["Force"], non_blocking=True)
        E_h.copy_(r["Etot"], non_blocking=True)
        V_h.copy_(r["Virial"], non_blocking=True)
        torch.cuda.current_stream().synchronize()

    for _ in range(max(3, args.warmup // 2)):
        e2e_step()
    e2e_steps = max(10, args.steps // 2)
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    t1 = time.perf_counter()
    barrier(ws)
    e2e_ms = max_over_ranks((t1 - t0) * 1e3 / e2e_steps, ws)
    h2d = frac_h.numel() * 8 + lat_h.numel() * 8
    d2h = F_h.numel() * F_h.element_size() + 8 + 72

    # ---- roofline of the dominant kernel
    per_kernel = {k: {"ms_per_launch": v[0] / v[1], "launches": v[1],
                      "share": None} for k, v in prof.items()}
    tot = sum(v[0] for v in prof.values())
    for k, v in prof.items():
        per_kernel[k]["share"] = v[0] / tot if tot else None
    dom = max(prof, key=lambda k: prof[k][0]) if prof else None
    es = 8 if prec == "float64" else 4
    S = 2 * M_NEIGH
    flops = {}
    for suf in ("", "_tc"):
        flops["dp_embed_bwd" + suf] = FLOP_EMB_BWD_PAIR * n_pairs
        flops["dp_embed_fwd" + suf] = FLOP_EMB_FWD_PAIR * n_pairs
        flops["dp_fit" + suf] = FLOP_FIT_ATOM * NATOMS
    # HBM-bound kernels: algorithmic bytes per launch (reads positions + types, writes the
    # block lengths and the occupied slots of list_neigh (int32) and ImageDR (4 values))
    hbm_bytes = {"nb_search": NATOMS * (24 + 4 + 4 * 2) + n_pairs * (4 + 4 * es)}
    peaks = {}
    pk_path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    src = "of measured (MEASURED_PEAKS.json)" if peaks else "of fallback"
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    simt_peak = sm_count() * 128 * 2 * sm_mhz * 1e6 / 1e12
    traffic = {}
    tp = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp))

    def roofline_of(k):
        t_launch = per_kernel[k]["ms_per_launch"] * 1e-3
        if k in hbm_bytes:
            ach = hbm_bytes[k] / t_launch / 1e9
            r = {"kernel": k, "bound": "hbm", "achieved": ach, "peak": hbm_peak,
                 "unit": "GB/s", "frac": ach / hbm_peak, "traffic": None,
                 "algorithmic_bytes_per_launch": hbm_bytes[k], "peak_source": src,
                 "limiter": "the FP64 pipe (65 % active in ncu: exact Fortran-order pair "
                            "arithmetic), not HBM; profiles/dp_tc_kernels_32k_full.md"}
        else:
            ach = flops[k] / t_launch / 1e12
            r = {"kernel": k, "bound": "tensor", "achieved": ach, "peak": bf16_peak,
                 "unit": "TFLOP/s", "frac": ach / bf16_peak, "traffic": None,
                 "algorithmic_flops_per_launch": flops[k], "peak_source": src + " bf16 burst",
                 "simt_fp32": {"achieved": ach, "peak_nominal_at_sm_clock": simt_peak,
                               "frac": ach / simt_peak}}
        tr = traffic.get(f"{k}:{prec}")
        if tr:
            r["traffic"] = tr["bytes_per_launch"]
            r["traffic_note"] = tr.get("note")
        return r

    roof = None
    if dom is not None and (dom in flops or dom in hbm_bytes):
        roof = roofline_of(dom)
        # the step's other main kernels, same arithmetic
        roof["others"] = {k: {q: v for q, v in roofline_of(k).items() if q != "kernel"}
                          for k in per_kernel if k != dom and (k in flops or k in hbm_bytes)}
    per_scope = {"nb_cells": 4, "dp_reduce": 2}
    launches = sum(v[1] * per_scope.get(k, 1) for k, v in prof.items())

    train_r = None
    if not args.no_train:
        train_r = run_train(args, ws, local, steps=20, warmup=3, plain_steps=3)
    md_r = None
    if not args.no_md:
        md_r = run_md(args, ws, local, steps=200)
    data_r = run_data(args, ws, local) if not args.no_data else None
    variants_r = run_dp_variants(args, ws, local) if not args.no_variants else None
    refops_r = calcops_reference_gpu(ln, dev) if not (args.no_variants or args.no_ref_gpu) \
        else None
    nep_train_r = None
    if not args.no_nep_train:
        nep_train_r = run_nep_train(args, ws, local, steps=10, warmup=3)
        if rank == 0 and not args.no_cpu_baseline:
            nep_train_r["cpu_baseline"] = cpu_baseline_nep_train(steps=3)
    lmp_r = None
    if not args.no_lammps:
        lmp_r, lmp_s, lmp_cfg = run_lammps(args, ws, local, steps=30, warmup=3)
        if rank == 0 and not args.no_cpu_baseline:
            lmp_r["cpu_baseline"] = cpu_baseline_lammps(lmp_s, lmp_cfg, [0, 1], NATOMS)
        del lmp_s
    nep = None
    if not args.no_nep:
        nep = run_nep(args, ws, local, steps=max(20, args.steps // 10), warmup=args.warmup,
                      sample_clocks=False)
        if rank == 0 and not args.no_cpu_baseline:
            nep["cpu_baseline"] = cpu_baseline_nep(steps=8, warmup=1)
    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline_run(steps=8, warmup=1)
    if rank != 0:
        return
    config = {"workload": "DP se_e2_a, 32,000-atom Li/Si (1:1) random-packed box, 0.05 atoms/A^3, "
                          "Rc 6.0, m=150/type (S=300), emb 25-25-25, M2 16, fit 50-50-50-1; "
                          "step = GPU neighbor search + E/F/V",
              "precision_form": prec, "natoms": NATOMS, "pairs": n_pairs,
              "parallelism": "replicas" if ws > 1 else "single GPU",
              "l2": "no flush: per-step working set ~230 MB (neighbor list + ImageDR) exceeds the "
                    "129 MB L2",
              "tile_tuning": tuning,
              "model_only_ms_per_step": model_ms,
              "model_only_value": ws * NATOMS / (model_ms * 1e-3), **acc}
    if plain64:
        config["plain_fp64"] = plain64
        if cb and cb.get("value"):
            config["plain_fp64"]["ratio_vs_cpu_baseline"] = plain64["value"] / cb["value"]
    if plain:
        config["plain_fp32"] = plain
        config["speedup_vs_plain_fp32"] = plain["ms_per_step"] / ms
        config["model_only_speedup_vs_plain_fp32"] = plain["model_only_ms_per_step"] / model_ms
    dtype = {"float32": "f32", "float64": "f64"}.get(prec, "bf16x3 tensor / f32 / f64 sums"
                                                     if prec != "mixed_fast" else "bf16 tensor / f32")
    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype, "data": "synthetic", "config": config,
            "e2e": {"value": ws * NATOMS / (e2e_ms * 1e-3), "unit": "atom-steps/s",
                    "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "kernels": per_kernel, "roofline": roof,
            "clocks": clocks, "cpu_baseline": cb, "nep": nep, "train": train_r, "md": md_r,
            "lammps": lmp_r, "nep_train": nep_train_r, "data_path": data_r,
            "dp_variants": variants_r, "reference_gpu_ops": refops_r}
    print(json.dumps(line))


def run_md_line(args, ws, rank, local):
    torch.cuda.set_device(local)
    from matpl_gb300 import _lib
    _lib.load()
    steps = args.steps if args.steps_given else 1000
    r = run_md(args, ws, local, steps)
    if rank != 0:
        return
    line = {"metric": r.pop("metric"), "value": r.pop("value"), "unit": r.pop("unit"),
            "n_gpus": ws, "steps": r.pop("steps"), "warmup": 2,
            "ms_per_step": r.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x3 tensor / f32 / f64 sums", "data": "synthetic", **r}
    print(json.dumps(line))


def run_train_line(args, ws, rank, local):
    torch.cuda.set_device(local)
    from matpl_gb300 import _lib
    _lib.load()
    steps = args.steps if args.steps_given else 30
    r = run_train(args, ws, local, steps=steps, warmup=args.warmup, plain_steps=5)
    if rank != 0:
        return
    line = {"metric": r.pop("metric"), "value": r.pop("value"), "unit": r.pop("unit"),
            "n_gpus": ws, "steps": r.pop("steps"), "warmup": r.pop("warmup"),
            "ms_per_step": r.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": r.pop("dtype"), "data": "synthetic", **r}
    print(json.dumps(line))


def run_nep_line(args, ws, rank, local):
    torch.cuda.set_device(local)
    from matpl_gb300 import _lib
    _lib.load()
    steps = args.steps if args.steps_given else 100
    r = run_nep(args, ws, local, steps=steps, warmup=args.warmup)
    if rank == 0 and not args.no_cpu_baseline:
        r["cpu_baseline"] = cpu_baseline_nep(steps=8, warmup=1)
    if rank != 0:
        return
    line = {"metric": r.pop("metric"), "value": r.pop("value"), "unit": r.pop("unit"),
            "n_gpus": ws, "steps": r.pop("steps"), "warmup": r.pop("warmup"),
            "ms_per_step": r.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": r.pop("dtype"), "data": "synthetic", **r}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed",
                    choices=["mixed", "mixed_tanhf", "mixed_fast", "float32", "float64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain-FP32 comparison run of a mixed form")
    ap.add_argument("--no-nep", action="store_true", help="skip the NEP workload")
    ap.add_argument("--no-train", action="store_true", help="skip the training-step workload")
    ap.add_argument("--no-md", action="store_true", help="skip the batched-replica MD workload")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the automatic tile shape of the mixed kernels (no autotuning)")
    ap.add_argument("--train-configs", type=int, default=TRAIN_CONFIGS,
                    help="configurations of the ragged training batch (64; fewer for captures)")
    ap.add_argument("--nep-atoms", type=int, default=NEP_NATOMS,
                    help="atoms of the NEP box (the benchmark is 100,000; smaller boxes of the "
                         "same density and model are for profiling captures)")
    ap.add_argument("--lammps-atoms", type=int, default=NATOMS,
                    help="local atoms of the LAMMPS pair-step box (32,000; smaller for captures)")
    ap.add_argument("--no-lammps", action="store_true", help="skip the LAMMPS pair-step workload")
    ap.add_argument("--lammps-access", default="auto", choices=["auto", "direct", "staged"],
                    help="how the LAMMPS driver reaches host arrays (profiling captures use "
                         "staged: ncu replays distort kernels that read host memory)")
    ap.add_argument("--nep-train-atoms", type=int, default=NEP_TRAIN_NATOMS,
                    help="atoms of the NEP training batch (20,000; smaller for captures)")
    ap.add_argument("--no-nep-train", action="store_true", help="skip the NEP training workload")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip the reference's own GPU code (comparator) beside the NEP step and "
                         "the CalcOps force / virial ops")
    ap.add_argument("--no-data", action="store_true", help="skip the data-path statistics pass")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the compressed / type-embedding DP variants")
    ap.add_argument("--workload", default="dp",
                    choices=["dp", "nep", "train", "md", "lammps", "neptrain"],
                    help="dp: the headline DP line (with a nep object); nep: the NEP line alone")
    argv = sys.argv[1:]
    args = ap.parse_args()
    args.steps_given = any(a.startswith("--steps") for a in argv)
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        ws = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, ws, rank)
        return
    ws, rank, local = dist_setup()
    if args.workload == "nep":
        run_nep_line(args, ws, rank, local)
        return
    if args.workload == "train":
        run_train_line(args, ws, rank, local)
        return
    if args.workload == "md":
        run_md_line(args, ws, rank, local)
        return
    if args.workload == "lammps":
        run_lammps_line(args, ws, rank, local)
        return
    if args.workload == "neptrain":
        run_nep_train_line(args, ws, rank, local)
        return
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
