"""The N > 1 replica path of bench.py on host ranks (gloo, world size 2): process-group setup
without a GPU, the barrier, the max-over-ranks step time and the whole-job value built from it,
and the reference arm's rank > 0 exit without work.  The path shards into independent replicas
(no collective on the data path), so these helpers are all of it."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    sys.argv = ["bench.py"]
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    t = bench.max_over_ranks(10.0 + rank, w)          # rank 1 is the slow one
    v = bench.replica_value(1000, bench.max_over_ranks(5.0 * (1 + rank), w), w)  # 5 / 10 ms
    q.put((r, w, dist.get_backend(), t, v))
    bench.barrier(w)
    dist.destroy_process_group()


def test_replica_helpers_on_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r, (rank, ws, backend, t, v) in enumerate(out):
        assert (rank, ws, backend) == (r, 2, "gloo")
        assert t == 11.0                               # max over ranks
        assert v == pytest.approx(2 * 1000 / 10e-3)    # all units / the slowest rank's time


def test_reference_arm_rank_above_zero_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "3",
                        "--warmup", "1"], cwd=REPO, env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_line_keeps_the_bench_contract():
    """Rank 0 of the reference arm prints one JSON line with the contract's keys, the requested
    step counts (warm-up at least 3), a host e2e object with no copies and a cpu_baseline that
    describes the same run."""
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "nep",
                        "--steps", "3", "--warmup", "3"], cwd=REPO, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["steps"] == 3 and d["warmup"] >= 3
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert "workload" in d["config"]
