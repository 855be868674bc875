"""bench.py's multi-GPU plumbing with two gloo ranks on the CPU: the barrier,
the gather, the whole-job throughput (all ranks' work over the slowest rank's
time), disjoint per-rank instance ranges, and the reference arm running on
rank 0 only."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, w = bench.init_dist()
    assert (r, w) == (rank, world)
    bench.barrier(w)
    # rank r "solved" 10 instances in (r + 1) seconds per step, 3 steps
    got = bench.gather(w, {"n": 10, "t": 3.0 * (r + 1)})
    lo, hi = bench.instance_range(r, 10, first=100)
    out = {"rank": r, "range": (lo, hi)}
    if r == 0:
        out["rate"], out["t_max"] = bench.job_throughput(got, "n", "t", 3)

    class A:
        config, warmup, steps, cpu_budget, tol = 0, 0, 1, 0.1, 1e-4
    out["ref_arm"] = bench.run_reference(A, r, w) if r != 0 else "rank0"
    q.put(out)
    dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    outs = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    by = {o["rank"]: o for o in outs}
    assert by[0]["range"] == (100, 110) and by[1]["range"] == (110, 120)
    # 20 instances per step over the slowest rank's 6 s for 3 steps
    assert by[0]["t_max"] == pytest.approx(6.0)
    assert by[0]["rate"] == pytest.approx(20 * 3 / 6.0)
    assert by[1]["ref_arm"] is None          # the reference arm runs on rank 0 only


class _StubBatch:
    """Stands in for PDHGBatch on a machine without a GPU: every instance
    'solved' at its planted optimum in 100 attempts, 50 ms per batched solve."""

    def __init__(self, problems, **kw):
        import sovereign_solver_gb300.workloads as wl
        self.problems = list(problems)
        self.seen = [p.name for p in self.problems]

    def solve_raw(self):
        from sovereign_solver_gb300 import _native as N
        st = N.BatchStats()
        st.solve_ms, st.lanes_per_column, st.blocks = 50.0, 1, 608
        return st

    def result(self, k):
        import numpy as np
        import sovereign_solver_gb300 as sps
        p = self.problems[k]
        k_seed = int(p.name.split("_")[1])
        import sovereign_solver_gb300.workloads as wl
        star = wl.batch_planted_lp(k_seed)[1]["obj_star"]
        return sps.SolveResult("optimal", np.zeros(p.n_vars), star, 100, y=np.zeros(p.n_eq), rel_kkt=5e-5)

    def close(self):
        pass


class _StubLib:
    """The C entry points the batched end-to-end leg calls, as no-ops; every
    other entry point is the real library's (option defaults, errors)."""

    def __init__(self, real):
        self._real = real

    def __getattr__(self, name):
        return getattr(self._real, name)

    def sps_batch_create(self, count, arr, opts, h):
        return 0

    def sps_batch_solve(self, h, st):
        return 0

    def sps_batch_get(self, h, k, x, y, r):
        return 0

    def sps_batch_destroy(self, h):
        return None


def _batch_rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import bench
    import sovereign_solver_gb300 as sps
    from sovereign_solver_gb300 import _native as N
    import torch.distributed as dist
    import test_multirank as me
    sps.PDHGBatch = me._StubBatch
    stub = me._StubLib(N.load())
    N.load = lambda: stub
    r, w = bench.init_dist()

    class A:
        batch, tol, max_iters, device, warmup, steps, e2e_steps = 3, 1e-4, 1000, 0, 1, 2, 1
        cpu_baseline = False
    try:
        q.put({"rank": r, "line": bench.run_batch(A, r, w)})
    except Exception:
        import traceback
        q.put({"rank": r, "error": traceback.format_exc()})
    dist.destroy_process_group()


def test_two_gloo_ranks_drive_the_batched_workload():
    """run_batch end to end on two ranks with a stub engine: each rank builds its
    own disjoint instance range, rank 0 alone reports, and the line counts both
    ranks' instances over the slowest rank's time."""
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_batch_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    outs = {o["rank"]: o for o in (q.get(timeout=300) for _ in procs)}
    for p in procs:
        p.join(timeout=60)
    assert all("error" not in o for o in outs.values()), [o.get("error") for o in outs.values()]
    assert all(p.exitcode == 0 for p in procs)
    assert outs[1]["line"] is None
    line = outs[0]["line"]
    assert line["n_gpus"] == 2 and line["optimal"] == 3       # rank 0's own instances
    # 2 ranks x 3 instances per step, 2 steps of 50 ms on the slowest rank
    assert line["value"] == pytest.approx(6 * 2 / 0.1)
    assert line["max_obj_error_vs_planted"] == 0.0
    assert line["config"]["workload"] == bench_workload(3)


def bench_workload(n):
    import bench
    return bench.batch_workload(n)


def test_gpus_flag_relaunches_as_ranks():
    """``bench.py --gpus 2`` outside torch.distributed relaunches itself as two
    ranks (torch.distributed.run, 127.0.0.1); rank 0 prints the one line."""
    import json
    import subprocess
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--impl", "reference",
           "--config", "0", "--steps", "3", "--warmup", "3", "--cpu-budget", "0.2"]
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    assert json.loads(lines[0])["n_gpus"] == 2
