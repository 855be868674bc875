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
