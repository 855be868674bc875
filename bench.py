"""Benchmark: restarted PDHG to 1e-4 relative KKT on one GB300.

Default workload: the synthetic transportation LP with 1000 sources x 2000
sinks (2M variables, 3000 rows, 4M nonzeros), solved from a cold start to a
relative KKT error of 1e-4 (FP32 iterates and SpMV, FP64 checks).  One step =
one complete solve.  ``value`` = solves/s with the problem resident in HBM
(``PDHGEngine.solve`` on the uploaded problem); ``e2e`` = the same through the
public C-ABI call from pinned host buffers (upload + layout + solve + solution
read-back inside the timed region).

The default run adds the metric's other parts as ``subrecords`` of the same
line, each with its own steps, clocks, roofline and CPU baseline: the power-law
LP (1M x 2M, ~21M nonzeros; SpMV rooflines of both passes), the batch of 4096
planted LPs (solves/s, p50/p99 attempts) and the learned warm start on 1000
held-out transportation seeds (warm batched against cold single-instance time
per solve).  ``--no-subrecords`` skips them.

``--impl reference`` times the reference algorithm (the oracle's C + OpenMP
restatement of ``solver/lp/pdhg.py``, all host threads) on the same workload;
both arms carry the same ``config`` dict.

Multi-GPU: replicas (each rank solves its own seed of the workload; no
collective), value = total solves / slowest rank's time.  ``--gpus N`` without
a torch.distributed environment relaunches the script as N ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sec & iters to 1e-4 rel KKT; solves/s batched; warm vs cold PDHG; SpMV % HBM"
TOL = 1e-4


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------- workloads
def make_workload(config: int, seed: int, powerlaw_nnz: int = 20_000_000):
    """The single-LP workloads.  ``powerlaw_nnz``: nonzero count the power-law
    LP's Zipf(1.5) row lengths are rescaled to; 0 keeps the lengths as drawn
    (clipped to [2, 5000]: about 1.1e8 nonzeros at m = 1M)."""
    import sovereign_solver_gb300.workloads as wl
    if config == 0:
        p, info = wl.planted_lp(seed=seed)
        return p, info, {"workload": "planted LP m=200 n=500 5% density u=2 (equality rows)", "seed": seed}
    if config == 1:
        p, info = wl.transportation_lp(1000, 2000, seed=seed)
        return p, info, {"workload": "transportation LP 1000 sources x 2000 sinks (n=2M, m=3000, nnz=4M)",
                         "seed": seed}
    if config == 2:
        p, info = wl.powerlaw_lp(seed=seed, target_nnz=powerlaw_nnz or None)
        rows = f"rescaled to ~{powerlaw_nnz / 1e6:g}M nnz" if powerlaw_nnz else "lengths as drawn"
        return p, info, {"workload": f"power-law LP m=1M n=2M Zipf(1.5) rows ({rows}), nnz={p.A_eq.nnz}",
                         "seed": seed}
    raise SystemExit(f"unknown config {config}")


def _batch_instance(k):
    import sovereign_solver_gb300.workloads as wl
    p, info = wl.batch_planted_lp(k)
    return p, info["obj_star"]


def make_batch(count: int, first: int):
    """Instances first .. first+count-1 of the batched workload, built in a
    spawn pool (deterministic per instance; outside every timed region)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    ks = list(range(first, first + count))
    workers = max(1, min(16, os.cpu_count() or 1))
    with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        out = list(ex.map(_batch_instance, ks, chunksize=32))
    return [o[0] for o in out], [o[1] for o in out]


def problem_bytes(p) -> int:
    """Host bytes one upload moves: CSR arrays of A_ub and A_eq plus c, b, lb, ub."""
    tot = 0
    for M in (p.A_ub, p.A_eq):
        tot += M.indptr.size * 4 + M.indices.size * 4 + M.data.size * 8
    return tot + 8 * (3 * p.n_vars + p.n_ineq + p.n_eq)


# dram__bytes_read.sum + dram__bytes_write.sum per launch of the iteration kernels,
# from one ncu capture per workload (seed 0, FP32 adaptive; --graph-mode 0 so the
# kernels are separate launches): the transportation LP 1000 x 2000 and the
# power-law LP rescaled to ~20M nonzeros.
MEASURED_TRAFFIC = {1: {"row": 40.44e6 + 0.00e6, "col": 64.88e6 + 1.20e6},
                    2: {"row": 189.54e6 + 7.03e6, "col": 228.30e6 + 16.03e6}}


def iteration_bytes(p) -> dict:
    """Algorithmic HBM bytes per launch of the two fused iteration kernels (FP32).

    row pass  (K x' + dual update):   8 nnz + 4(m+1) + 4n + 20m
    col pass  (K^T y' + primal update + averages):
              8 nnz + 4(n+1) + 4m + 28n (+8n with per-column bounds) + 16m
    Vectors gathered through the SpMV are counted once (L2-resident gather).
    """
    n, m = p.n_vars, p.n_ineq + p.n_eq
    nnz = p.A_ub.nnz + p.A_eq.nnz
    lb, ub = np.asarray(p.lb), np.asarray(p.ub)
    uniform = (np.all(lb == lb[0]) and np.all(ub == ub[0]) and (lb[0] == 0 or np.isinf(lb[0]))
               and np.isinf(ub[0]) and ub[0] > 0)
    row = 8 * nnz + 4 * (m + 1) + 4 * n + 20 * m
    col = 8 * nnz + 4 * (n + 1) + 4 * m + 28 * n + (0 if uniform else 8 * n) + 16 * m
    spmv_row = 8 * nnz + 4 * (m + 1) + 4 * n + 4 * m
    spmv_col = 8 * nnz + 4 * (n + 1) + 4 * m + 4 * n
    return {"row": row, "col": col, "spmv_row": spmv_row, "spmv_col": spmv_col, "nnz": nnz}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# --------------------------------------------------------------------------- CPU reference timing
def reference_sample(p, budget_s: float):
    """Time the reference algorithm (C + OpenMP restatement) on a bounded number
    of iterations; returns dict with seconds per iteration and the sample."""
    from oracle import pdhg_ref, pdhg_ref_c
    t0 = time.perf_counter()
    std = pdhg_ref.to_standard_form(p)
    t_std = time.perf_counter() - t0
    # probe with a few iterations, then size the sample to the budget
    t0 = time.perf_counter()
    pdhg_ref_c.solve_std(std, 5, 0.0)
    probe = (time.perf_counter() - t0) / 5
    iters = int(max(10, min(100000, budget_s / max(probe, 1e-6))))
    t0 = time.perf_counter()
    pdhg_ref_c.solve_std(std, iters, 0.0)
    dt = time.perf_counter() - t0
    return {"s_per_iter": dt / iters, "iters": iters, "seconds": dt, "std_form_s": t_std,
            "threads": pdhg_ref_c.threads()}


def reference_gpu_path(p, iters: int = 300):
    """The reference's own GPU path (``solver/lp/pdhg_gpu.py:315-443``: torch-CUDA
    FP64 sparse CSR, host KKT check every 50 iterations), unmodified, from its
    install in baseline/_ref, on the same LP: seconds per iteration as the
    difference of a short and a long capped run (setup excluded).  A reported
    secondary figure; the reference arm's value stays the CPU path."""
    ref = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref, "solver")):
        return {"unavailable": "the reference is not installed in baseline/_ref"}
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "torch sees no CUDA device"}
    except ImportError:
        return {"unavailable": "torch is not importable"}
    if ref not in sys.path:
        sys.path.insert(0, ref)
    from solver.lp.pdhg_gpu import DeviceEngine, solve_lp_pdhg_gpu
    from solver.problem import Problem as RefProblem
    rp = RefProblem(c=np.asarray(p.c, float), A_ub=p.A_ub, b_ub=np.asarray(p.b_ub, float), A_eq=p.A_eq,
                    b_eq=np.asarray(p.b_eq, float), lb=np.asarray(p.lb, float), ub=np.asarray(p.ub, float),
                    integer_mask=np.zeros(p.n_vars, dtype=bool))
    backend = DeviceEngine(device="cuda").backend
    short = max(50, iters // 3)

    def timed(k):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = solve_lp_pdhg_gpu(rp, device="cuda", max_iters=k)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, r
    timed(short)                                 # warm-up: torch / cuSPARSE initialisation
    t_s, _ = timed(short)
    t_l, r = timed(iters)
    return {"s_per_iter": (t_l - t_s) / (iters - short), "backend": backend, "dtype": "fp64",
            "sample": (f"solve_lp_pdhg_gpu(device='cuda') capped at {short} and {iters} iterations, "
                       f"per-iteration time = difference / {iters - short} (standard form, upload and "
                       f"setup cancel); status at the cap {r.status!r}"),
            "torch": torch.__version__}


def load_reference_iterations(config: int):
    path = os.path.join(ROOT, "tests", "golden", "reference_iterations.json")
    try:
        with open(path) as f:
            return json.load(f).get(str(config))
    except OSError:
        return None


# --------------------------------------------------------------------------- arms
def run_ours(args, rank, world):
    import ctypes as C
    import sovereign_solver_gb300 as sps
    from sovereign_solver_gb300 import _native as N, pdhg

    p, info, cfg = make_workload(args.config, seed=args.seed + rank, powerlaw_nnz=args.powerlaw_nnz)
    hbm, peak_kind = peaks()
    form = kkt_form_of(args)
    eng = sps.PDHGEngine(p, tol=args.tol, max_iters=args.max_iters, device=args.device,
                         graph_mode=args.graph_mode, kkt_form=form)
    for _ in range(args.warmup):
        r = eng.solve_raw()
    flush = None
    if args.config == 0:          # the planted LP fits in L2: overwrite L2 between timed solves
        import torch
        flush = torch.empty(64 << 20, dtype=torch.int32, device=f"cuda:{args.device}")
    barrier(world)
    ms, iters, res = [], [], None
    t_wall = time.perf_counter()
    with ClockSampler(args.device) as clk:
        for _ in range(args.steps):
            if flush is not None:
                flush.zero_()
                torch.cuda.synchronize(args.device)
            r = eng.solve_raw()
            ms.append(r.solve_ms)
            iters.append(r.iterations)
            res = r
    wall = time.perf_counter() - t_wall
    x, y = eng.solution()
    launches = int(res.kernel_launches) * args.steps
    kt, kg = np.zeros(3), np.zeros(3)
    N.check(eng.lib.sps_time_iteration_kernels(eng.h, 20, N.f64p(kt)), eng.h)         # host launches
    N.check(eng.lib.sps_time_iteration_kernels_graph(eng.h, 20, N.f64p(kg)), eng.h)   # as in the solve's graph
    eng.close()

    # end to end: public C-ABI call from pinned host buffers
    d = pdhg._Desc(p)
    lib = N.load()
    pinned, seen = [], set()
    for a in d.arrays():          # one registration per buffer (builders may share arrays)
        if a.size and a.ctypes.data not in seen and lib.sps_pin_host(a.ctypes.data, a.nbytes) == 0:
            pinned.append(a)
            seen.add(a.ctypes.data)
    opts = pdhg.make_options(tol=args.tol, max_iters=args.max_iters, device=args.device,
                             graph_mode=args.graph_mode, kkt_form=form)
    xo, yo = np.empty(d.n), np.empty(d.m_ub + d.m_eq)
    for a in (xo, yo):
        if lib.sps_pin_host(a.ctypes.data, a.nbytes) == 0:
            pinned.append(a)
    e2e_s = []
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    for it in range(e2e_steps + 1):
        t0 = time.perf_counter()
        h = C.c_void_p()
        N.check(lib.sps_create(C.byref(d.desc), C.byref(opts), C.byref(h)), None)
        rr = N.Result()
        N.check(lib.sps_solve(h, C.byref(rr)), h)
        N.check(lib.sps_get_solution(h, N.f64p(xo), N.f64p(yo)), h)
        lib.sps_destroy(h)
        if it > 0:                      # first call pays one-time lazy CUDA init
            e2e_s.append(time.perf_counter() - t0)
    for a in pinned:
        lib.sps_unpin_host(a.ctypes.data)

    per_rank = {"ms": sum(ms), "e2e_s": sum(e2e_s), "e2e_steps": len(e2e_s), "n": 1}
    gathered = gather(world, per_rank)
    if rank != 0:
        return None
    value, t_max = job_throughput(gathered, "n", "ms", args.steps, 1e-3)
    e2e_t = max(g["e2e_s"] / g["e2e_steps"] for g in gathered)
    ib = iteration_bytes(p)
    dom = "col" if kg[1] >= kg[0] else "row"
    dom_ms = kg[1] if dom == "col" else kg[0]
    achieved = ib[dom] / (dom_ms / 1e3) / 1e9
    status = N.STATUS.get(res.status, str(res.status))
    it_med = int(np.median(iters))
    line = {
        "metric": METRIC,
        "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic",
        "config": {**cfg, "tol_rel_kkt": args.tol},
        "mode": "adaptive", "precision": "fp32 iterates, fp64 checks (fp64 continuation if fp32 stalls)",
        "parallelism": f"replicas x{world}",
        "l2": ("working set < 129 MB L2: a 256 MB buffer is written before each timed solve" if flush is not None
               else "working set > 129 MB L2 (inputs larger than L2)"),
        "kkt_form": form,
        "iters_to_tol": it_med,
        "sec_to_tol": t_max / args.steps,
        "s_per_iter": t_max / args.steps / max(it_med, 1),
        "status": status, "rel_kkt": float(res.rel_kkt), "rel_kkt_lagrangian": float(res.rel_kkt_lagrangian),
        "escalated_fp64": bool(res.escalated),
        "obj_error": objective_error(args.config, args.seed + rank, float(res.objective), info),
        "restarts": int(res.restarts), "setup_ms": float(res.setup_ms),
        "host_wall_s_timed": wall,
        "gpu_launches": launches,
        "e2e": {"value": world / e2e_t, "unit": "solves/s", "sec_per_solve": e2e_t,
                "h2d_bytes_per_step": problem_bytes(p), "d2h_bytes_per_step": 8 * (len(x) + len(y))},
        "kernel_ms": {"row_pass": kg[0], "col_pass": kg[1], "accept_rate": kg[2],
                      "timing": ("in-graph: events around replays of a graph of 20 x [row, column] passes and of one "
                                 "of 20 x [row] passes; column = the difference"),
                      "host_launched": {"row_pass": kt[0], "col_pass": kt[1]}},
        "attempt": {"us_in_graph": (kg[0] + kg[1]) * 1e3,
                    "gbs": (ib["row"] + ib["col"]) / ((kg[0] + kg[1]) / 1e3) / 1e9,
                    "frac": (ib["row"] + ib["col"]) / ((kg[0] + kg[1]) / 1e3) / 1e9 / hbm},
        "roofline": {"bound": "hbm", "kernel": f"ad_{dom}_step (fused {'CSC' if dom == 'col' else 'CSR'} SpMV + update)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "algorithmic_bytes": ib[dom],
                     "traffic": (MEASURED_TRAFFIC.get(args.config, {}).get(dom)
                                 if args.seed == 0 and (args.config != 2 or args.powerlaw_nnz == 20_000_000)
                                 else None),
                     "other_pass_gbs": (ib["row" if dom == "col" else "col"] /
                                        ((kg[0] if dom == "col" else kg[1]) / 1e3) / 1e9)},
        "clocks": clk.summary(),
    }
    if args.config == 2:
        # the row pass's random gathers against the floor of a pass with random indices
        # over a vector of n entries (same nonzeros, nothing else in the kernel)
        gf = np.zeros(2)
        N.check(N.load().sps_time_gather_floor(int(ib["nnz"]), int(p.n_vars), 20, args.device, N.f64p(gf)), None)
        line["gather_floor"] = {
            "random_ms": gf[0], "in_order_ms": gf[1], "nnz": int(ib["nnz"]), "vector": int(p.n_vars),
            "row_pass_over_random_floor": kt[0] / gf[0],
            "what": ("sps_time_gather_floor: 16-byte index and value loads, 4 gathers per thread, nothing else; "
                     "random = uniform column indices, in_order = the same bytes with indices walking x")}
    # whole solve: both passes' algorithmic bytes per attempt x attempts / solve time (the checks,
    # one per 64 attempts, move more bytes that are not counted)
    line["solve_avg_gbs"] = (ib["row"] + ib["col"]) * it_med / (t_max / args.steps) / 1e9
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(p, args)
    return line


def kkt_form_of(args) -> str:
    """The error form the engine terminates on: the Lagrangian form by default;
    the PDLP form on the power-law LP, whose 10-wide bounds far from x* put the
    Lagrangian dual bound at a relative gap that FP32 iterates cannot close."""
    if args.kkt_form != "auto":
        return args.kkt_form
    return "pdlp" if args.config == 2 else "lagrangian"


def objective_error(config: int, seed: int, objective: float, info: dict):
    """|objective - optimum| / (1 + |optimum|) against the planted optimum or the
    exact optimum committed with the fixtures (HiGHS dual simplex), else None."""
    if "obj_star" in info:
        opt, src = info["obj_star"], "planted optimum c^T x* = b^T y*"
    else:
        key = {1: f"transport_1000x2000_s{seed}", 4: f"transport_family_200x400_s{seed}"}.get(config)
        try:
            with open(os.path.join(ROOT, "tests", "golden", "optima.json")) as f:
                entry = json.load(f)[key]
        except (OSError, KeyError, TypeError, ValueError):
            return None
        opt, src = float(entry["objective"]), f"exact optimum ({entry['solver']}, tests/golden/optima.json)"
    return {"value": abs(objective - opt) / (1 + abs(opt)), "objective": objective, "optimum": opt, "against": src}


def _ref_solve_one(k):
    """Worker (spawned, one OpenMP thread): the reference algorithm on batched instance k."""
    os.environ["OMP_NUM_THREADS"] = "1"
    import sovereign_solver_gb300.workloads as wl
    from oracle import pdhg_ref_c
    p = wl.batch_planted_lp(k)[0]
    t0 = time.perf_counter()
    r = pdhg_ref_c.solve(p, max_iters=100000, tol=1e-4)
    return k, r.status, r.iterations, time.perf_counter() - t0


def batch_cpu_baseline(args):
    """Reference algorithm (C restatement of solver/lp/pdhg.py, one thread per
    process) on every 128th instance of the batch (32 LPs), one spawned process
    per host core; solves/s = 32 / wall time."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    ks = list(range(0, 4096, 128))
    procs = max(1, min(16, os.cpu_count() or 1))
    t0 = time.perf_counter()
    with ProcessPoolExecutor(procs, mp_context=mp.get_context("spawn")) as ex:
        out = list(ex.map(_ref_solve_one, ks))
    wall = time.perf_counter() - t0
    per = [o[3] for o in out]
    return {"value": len(ks) / wall, "unit": "solves/s", "cores": procs, "kind": "port",
            "sample": (f"reference algorithm (C restatement of solver/lp/pdhg.py) to 1e-4 on instances "
                       f"0, 128, ..., 3968 of the batch ({len(ks)} LPs), {procs} single-threaded processes, "
                       f"{wall:.1f} s wall; per-LP {np.median(per):.2f} s median, "
                       f"{sum(o[1] == 'optimal' for o in out)}/{len(ks)} optimal"),
            "serial_s_per_solve": float(np.mean(per)),
            "one_core_value": 1.0 / float(np.mean(per))}     # solves/s of one single-threaded process


def run_batch(args, rank, world):
    """Batched workload: ``--batch`` LPs of the config-0 construction with m
    log-uniform in [50, 5000], n = m * U[1.5, 3], 10-50 nonzeros per column,
    solved to 1e-4 in one persistent launch.  One step = one batched solve of
    every instance on the resident batch (graph replay); value = solves/s.
    e2e = sps_batch_create + sps_batch_solve + sps_batch_get of every instance
    from host arrays.  Multi-GPU: replicas, each rank its own instance range."""
    import ctypes as C
    import sovereign_solver_gb300 as sps
    from sovereign_solver_gb300 import _native as N, pdhg

    t = time.perf_counter()
    probs, stars = make_batch(args.batch, first=instance_range(rank, args.batch)[0])
    log(f"generated {len(probs)} instances in {time.perf_counter() - t:.1f}s")
    nnz = [p.A_eq.nnz + p.A_ub.nnz for p in probs]
    hbm, peak_kind = peaks()
    b = sps.PDHGBatch(probs, tol=args.tol, max_iters=args.max_iters, device=args.device)
    for _ in range(args.warmup):
        b.solve_raw()
    barrier(world)
    ms, st = [], None
    with ClockSampler(args.device) as clk:
        for _ in range(args.steps):
            st = b.solve_raw()
            ms.append(st.solve_ms)
    res = [b.result(k) for k in range(len(probs))]
    its = np.array([r.iterations for r in res])
    kkts = np.array([r.rel_kkt for r in res])
    obj_err = max(abs(r.objective - s_) / (1 + abs(s_)) for r, s_ in zip(res, stars))
    # algorithmic bytes of the persistent launch: per attempt and instance the
    # row pass (8 nnz + 4(m+1) + 4n + 20m) and the column pass (8 nnz + 4(n+1) +
    # 4m + 36n + 16m) -- the single-LP model with per-column bounds
    alg = 0.0
    for p, r in zip(probs, res):
        n_, m_ = p.n_vars, p.n_ineq + p.n_eq
        z = p.A_eq.nnz + p.A_ub.nnz
        alg += r.iterations * (16 * z + 4 * (m_ + 1) + 4 * n_ + 20 * m_ + 4 * (n_ + 1) + 4 * m_ + 36 * n_ + 16 * m_)
    lanes, blocks, esc, hand = st.lanes_per_column, st.blocks, st.escalated, st.handed_off
    b.close()

    # end to end through the C ABI from host arrays
    descs = [pdhg._Desc(p) for p in probs]
    arr = (N.ProblemDesc * len(descs))(*[d.desc for d in descs])
    lib = N.load()
    opts = pdhg.make_options(tol=args.tol, max_iters=args.max_iters, device=args.device)
    xs = [np.empty(p.n_vars) for p in probs]
    ys = [np.empty(p.n_ineq + p.n_eq) for p in probs]
    e2e_s = []
    for it in range(max(1, args.e2e_steps)):
        t0 = time.perf_counter()
        h = C.c_void_p()
        N.check(lib.sps_batch_create(len(descs), arr, C.byref(opts), C.byref(h)), None)
        sst = N.BatchStats()
        rc = lib.sps_batch_solve(h, C.byref(sst))
        rr = N.Result()
        for k in range(len(descs)):
            rc = rc or lib.sps_batch_get(h, k, N.f64p(xs[k]), N.f64p(ys[k]), C.byref(rr))
        lib.sps_batch_destroy(h)
        if rc:
            raise RuntimeError(f"batched e2e failed: {rc}")
        e2e_s.append(time.perf_counter() - t0)

    per_rank = {"ms": sum(ms), "e2e_s": sum(e2e_s) / len(e2e_s), "n": len(probs)}
    gathered = gather(world, per_rank)
    if rank != 0:
        return None
    value, t_max = job_throughput(gathered, "n", "ms", args.steps, 1e-3)
    total = sum(g["n"] for g in gathered)
    e2e_t = max(g["e2e_s"] for g in gathered)
    achieved = alg / (t_max / args.steps) / 1e9
    line = {
        "metric": METRIC,
        "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic",
        "config": {"workload": batch_workload(args.batch), "tol_rel_kkt": args.tol},
        "total_nnz": int(sum(nnz)),
        "mode": "adaptive, one persistent launch (graph replay)",
        "precision": "fp32 iterates, fp64 checks, fp64 continuation of stalled instances",
        "parallelism": f"replicas x{world}", "l2": "working set > 129 MB L2 (inputs larger than L2)",
        "iters_p50": float(np.percentile(its, 50)), "iters_p99": float(np.percentile(its, 99)),
        "iters_max": int(its.max()), "optimal": int(sum(r.status == "optimal" for r in res)),
        "escalated_fp64": int(esc), "handed_off": int(hand),
        "max_rel_kkt": float(kkts.max()), "max_obj_error_vs_planted": float(obj_err),
        "lanes_per_column": int(lanes), "persistent_blocks": int(blocks),
        "gpu_launches": 3 * args.steps,
        "e2e": {"value": total / e2e_t, "unit": "solves/s", "sec_per_batch": e2e_t,
                "h2d_bytes_per_step": int(sum(problem_bytes(p) for p in probs)),
                "d2h_bytes_per_step": int(sum(8 * (p.n_vars + p.n_ineq + p.n_eq) for p in probs))},
        "roofline": {"bound": "hbm", "kernel": "k_batch_solve (persistent, whole PDHG loop per instance)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "algorithmic_bytes": alg, "traffic": None},
        "clocks": clk.summary(),
    }
    if args.cpu_baseline:
        line["cpu_baseline"] = batch_cpu_baseline(args)
    return line


def batch_workload(count: int) -> str:
    return (f"batched: {count} planted LPs per GPU (seeds = instance index), m log-uniform [50,5000], "
            f"n = m*U[1.5,3], 10-50 nnz/column, u=2")


WEIGHTS = os.path.join(ROOT, "sovereign-solver_gb300", "data", "warmstart_transport_200x400.npz")
TEST_SEED0 = 10_000_000          # held-out seeds (training used 0 .. 19 999)


def run_warmstart(args, rank, world):
    """Learned warm start on the 200 x 400 transportation family: ``--batch``
    held-out seeds (per GPU).  One step = GNN inference on the device straight
    into the batch's warm-start buffers + one batched solve of every seed,
    batch resident; value = solves/s.  Reported beside it: the same batch solved cold, and cold
    single-instance PDHG (create + solve + read-back per LP) on a sample.
    e2e = sps_batch_create + inference + warm starts + solve + read-back of
    every instance from host arrays."""
    import ctypes as C
    import sovereign_solver_gb300 as sps
    from sovereign_solver_gb300 import _native as N
    from sovereign_solver_gb300.gnn import WarmStartGNN
    from sovereign_solver_gb300.warmstart import transport_instances
    from sovereign_solver_gb300.workloads import TransportFamily

    fam = TransportFamily()
    template = fam.problem(0)
    seeds = np.arange(*instance_range(rank, args.batch, TEST_SEED0))
    probs = transport_instances(fam, template, seeds)
    net = WarmStartGNN.load(WEIGHTS, template, max_batch=16, device=args.device)
    hbm, peak_kind = peaks()
    b = sps.PDHGBatch(probs, tol=args.tol, max_iters=args.max_iters, device=args.device)
    # cold batched (resident)
    b.set_warm_starts(None)
    for _ in range(max(1, args.warmup // 2)):
        b.solve_raw()
    t_cold = []
    for _ in range(max(1, args.steps // 2)):
        st = b.solve_raw()
        t_cold.append(st.solve_ms / 1e3)
    cold = [b.result(k) for k in range(len(probs))]
    # warm batched (resident): inference + warm starts + solve
    def warm_step():
        t0 = time.perf_counter()
        b.set_warm_starts_gnn(net)              # inference on the device into the batch's buffers
        t1 = time.perf_counter()
        st = b.solve_raw()
        return t1 - t0, st.solve_ms / 1e3, time.perf_counter() - t0
    for _ in range(args.warmup):
        warm_step()
    barrier(world)
    steps = []
    with ClockSampler(args.device) as clk:
        for _ in range(args.steps):
            steps.append(warm_step())
    warm = [b.result(k) for k in range(len(probs))]
    b.close()
    # cold single-instance PDHG on a sample (create + solve + read-back)
    single = []
    for p in probs[:args.single_sample]:
        t0 = time.perf_counter()
        with sps.PDHGEngine(p, tol=args.tol, max_iters=args.max_iters, device=args.device) as eng:
            r = eng.solve()
        single.append((time.perf_counter() - t0, r.iterations, r.status == "optimal"))
    # end to end through the C ABI from host arrays (create, inference, warm starts, solve, read-back)
    from sovereign_solver_gb300 import pdhg
    descs = [pdhg._Desc(p) for p in probs]
    arr = (N.ProblemDesc * len(descs))(*[d.desc for d in descs])
    lib = N.load()
    opts = pdhg.make_options(tol=args.tol, max_iters=args.max_iters, device=args.device)
    xs = [np.empty(p.n_vars) for p in probs]
    ys = [np.empty(p.n_ineq + p.n_eq) for p in probs]
    scales = np.array([net.scales[k] for k in ("c", "b", "x", "y")], dtype=np.float64)
    e2e_s = []
    for _ in range(max(1, args.e2e_steps)):
        t0 = time.perf_counter()
        h = C.c_void_p()
        N.check(lib.sps_batch_create(len(descs), arr, C.byref(opts), C.byref(h)), None)
        rc = lib.sps_batch_set_warm_starts_gnn(h, net.h, N.f64p(scales))
        sst = N.BatchStats()
        rc = rc or lib.sps_batch_solve(h, C.byref(sst))
        rr = N.Result()
        for k in range(len(descs)):
            rc = rc or lib.sps_batch_get(h, k, N.f64p(xs[k]), N.f64p(ys[k]), C.byref(rr))
        lib.sps_batch_destroy(h)
        if rc:
            raise RuntimeError(f"warm-start e2e failed: {rc}")
        e2e_s.append(time.perf_counter() - t0)
    net.close()

    per_rank = {"t": sum(s_[2] for s_ in steps), "e2e": sum(e2e_s) / len(e2e_s), "n": len(probs)}
    gathered = gather(world, per_rank)
    if rank != 0:
        return None
    value, t_max = job_throughput(gathered, "n", "t", args.steps)
    total = sum(g["n"] for g in gathered)
    ci = np.array([r.iterations for r in cold])
    wi = np.array([r.iterations for r in warm])
    nnz = probs[0].A_ub.nnz + probs[0].A_eq.nnz
    n_, m_ = probs[0].n_vars, probs[0].n_ineq + probs[0].n_eq
    per_it = 16 * nnz + 4 * (m_ + 1) + 4 * n_ + 20 * m_ + 4 * (n_ + 1) + 4 * m_ + 28 * n_ + 16 * m_
    solve_s = np.mean([s_[1] for s_ in steps])
    achieved = float(wi.sum()) * per_it / solve_s / 1e9
    # per chunk of 16 instances: 2 LP-feature kernels + 19 network kernels (L = 3) +
    # the batch's input and output kernels; per step 3 batch kernels
    fwd_launches = 9 + 4 * net.layers + 2
    line = {
        "metric": METRIC,
        "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic",
        "config": {"workload": warmstart_workload(args.batch), "tol_rel_kkt": args.tol},
        "mode": "GNN inference + warm-started batched PDHG (cold fallback on)",
        "precision": "fp32 iterates, fp64 checks; GNN bf16 weights, fp32 accumulation",
        "parallelism": f"replicas x{world}", "l2": "working set > 129 MB L2 (inputs larger than L2)",
        "warm_iters_median": float(np.median(wi)), "cold_iters_median": float(np.median(ci)),
        "warm_iters_mean": float(wi.mean()), "cold_iters_mean": float(ci.mean()),
        "warm_used": int(sum(r.stats["warm_start_used"] for r in warm)),
        "warm_optimal": int(sum(r.status == "optimal" for r in warm)),
        "cold_optimal": int(sum(r.status == "optimal" for r in cold)),
        "max_rel_kkt_warm": float(max(r.rel_kkt for r in warm)),
        "gnn_inference_s_per_solve": float(np.mean([s_[0] for s_ in steps])) / len(probs),
        "warm_batched_s_per_solve": t_max / args.steps / total * world,
        "cold_batched_s_per_solve": float(np.mean(t_cold)) / len(probs),
        "cold_single_s_per_solve": float(np.mean([s_[0] for s_ in single])),
        "cold_single_iters_median": float(np.median([s_[1] for s_ in single])),
        "cold_single_sample": len(single),
        "gpu_launches": args.steps * (3 + fwd_launches * ((len(probs) + 15) // 16)),
        "e2e": {"value": total / max(g["e2e"] for g in gathered), "unit": "solves/s",
                "sec_per_batch": max(g["e2e"] for g in gathered),
                "h2d_bytes_per_step": int(sum(problem_bytes(p) for p in probs)),
                "d2h_bytes_per_step": int(sum(8 * (p.n_vars + p.n_ineq + p.n_eq) for p in probs))},
        "roofline": {"bound": "hbm", "kernel": "k_batch_solve (persistent, warm-started)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "algorithmic_bytes": float(wi.sum()) * per_it, "traffic": None},
        "clocks": clk.summary(),
    }
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(probs[0], args, ref_key=f"4:{TEST_SEED0}")
    return line


def warmstart_workload(count: int) -> str:
    return (f"learned warm start: transportation family 200x400 (n=80k, m=600, nnz=160k), "
            f"{count} held-out seeds per GPU from {TEST_SEED0}, network trained on seeds 0..19999")


def branching_node(args, rank, on_cpu=False):
    """Config 5: the set-covering MILP node, its LP relaxation (solved to 1e-6 on
    the GPU, or by the oracle's simplex for the CPU reference arm; outside every
    timed region), the strong-branching candidates and the 2K child problems
    (down_0, up_0, down_1, ...)."""
    import sovereign_solver_gb300 as sps
    import sovereign_solver_gb300.branching as br
    import sovereign_solver_gb300.workloads as wl
    p, _ = wl.set_cover_milp(seed=args.seed + rank)
    relax = sps.Problem(c=p.c, A_ub=p.A_ub, b_ub=p.b_ub, A_eq=p.A_eq, b_eq=p.b_eq, lb=p.lb, ub=p.ub,
                        integer_mask=np.zeros(p.n_vars, dtype=bool))
    if on_cpu:
        from oracle import simplex
        r = simplex.solve(relax)
        lp = sps.SolveResult(r.status, r.x, r.objective, r.iterations, y=np.zeros(p.n_ineq + p.n_eq))
    else:
        lp = sps.solve_lp_pdhg(relax, tol=1e-6, device=args.device)
    top = br.strong_candidates(lp.x, p.integer_mask)
    kids = []
    for j in top:
        kids.append(br.child_problem(p, p.lb, p.ub, int(j), "down", lp.x[j]))
        kids.append(br.child_problem(p, p.lb, p.ub, int(j), "up", lp.x[j]))
    return p, lp, top, kids


def branching_cpu_baseline(kids, parent_obj, budget_s):
    """The reference's _lp_gain loop (one simplex solve per child,
    solver/milp/branching.py:132-144, 187-188) with the oracle's FP64 bounded
    revised simplex, over as many children as the budget allows (at least one)."""
    from oracle import simplex
    t0 = time.perf_counter()
    done = 0
    for kp in kids:
        simplex.solve(kp)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "child LPs/s", "cores": 1, "kind": "port",
            "sample": (f"{done} of the {len(kids)} children solved one after another by the oracle's FP64 "
                       f"bounded revised simplex in {dt:.1f} s (the reference's strong branching calls its "
                       f"own simplex once per child, solver/milp/branching.py:132-144)")}


def run_branching(args, rank, world):
    """Strong branching at a MILP node: the 2K = 40 child LPs of the 20 most
    fractional variables of a 200 x 2000 set-covering node, solved
    to 1e-4 in one batched launch, each warm-started from the parent's point.
    One step = one batched solve of the resident children (graph replay);
    value = child LPs/s.  e2e = ``branching.child_gains`` from host arrays
    (children built, batch created, warm starts uploaded, solved, read back)."""
    import sovereign_solver_gb300 as sps
    import sovereign_solver_gb300.branching as br
    p, lp, top, kids = branching_node(args, rank)
    hbm, peak_kind = peaks()
    starts = [(np.clip(lp.x, k.lb, k.ub), lp.y, None) for k in kids]
    b = sps.PDHGBatch(kids, tol=args.tol, max_iters=args.max_iters, device=args.device)
    b.set_warm_starts(starts)
    for _ in range(args.warmup):
        b.solve_raw()
    barrier(world)
    ms, st = [], None
    with ClockSampler(args.device) as clk:
        for _ in range(args.steps):
            st = b.solve_raw()
            ms.append(st.solve_ms)
    res = [b.result(k) for k in range(len(kids))]
    team, blocks = st.team, st.blocks
    b.close()
    its = np.array([r.iterations for r in res])
    alg = 0.0
    for kp, r in zip(kids, res):
        n_, m_, z = kp.n_vars, kp.n_ineq + kp.n_eq, kp.A_ub.nnz + kp.A_eq.nnz
        alg += r.iterations * (16 * z + 4 * (m_ + 1) + 4 * n_ + 20 * m_ + 4 * (n_ + 1) + 4 * m_ + 36 * n_ + 16 * m_)
    gains = np.array([br.gain_of(r, lp.objective) for r in res])
    e2e_s = []
    for _ in range(max(1, args.e2e_steps)):
        t0 = time.perf_counter()
        br.child_gains(p, top, lp.x, p.lb, p.ub, lp.objective, y=lp.y, tol=args.tol,
                       max_iters=args.max_iters, device=args.device)
        e2e_s.append(time.perf_counter() - t0)
    per_rank = {"ms": sum(ms), "e2e_s": sum(e2e_s) / len(e2e_s), "n": len(kids)}
    gathered = gather(world, per_rank)
    if rank != 0:
        return None
    value, t_max = job_throughput(gathered, "n", "ms", args.steps, 1e-3)
    total = sum(g["n"] for g in gathered)
    e2e_t = max(g["e2e_s"] for g in gathered)
    achieved = alg / (t_max / args.steps) / 1e9
    nz = p.A_ub.nnz
    line = {
        "metric": METRIC, "value": value, "unit": "child LPs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic",
        "config": {"workload": BRANCH_WORKLOAD, "tol_rel_kkt": args.tol},
        "nnz": int(nz),
        "mode": "adaptive batched, warm-started from the parent LP",
        "precision": "fp32 iterates, fp64 checks, fp64 continuation of stalled instances",
        "parallelism": f"replicas x{world}",
        "l2": "working set < 129 MB L2 (the 40 children's matrices, 1.3 MB, stay in L2)",
        "iters_p50": float(np.percentile(its, 50)), "iters_max": int(its.max()),
        "statuses": {s_: int(sum(r.status == s_ for r in res)) for s_ in sorted({r.status for r in res})},
        "infinite_gains": int(np.isinf(gains).sum()), "team": int(team), "persistent_blocks": int(blocks),
        "parent_rel_kkt": float(lp.rel_kkt),
        "gpu_launches": 3 * args.steps,
        "e2e": {"value": total / e2e_t, "unit": "child LPs/s", "sec_per_node": e2e_t,
                "h2d_bytes_per_step": int(sum(problem_bytes(k) for k in kids)),
                "d2h_bytes_per_step": int(sum(8 * (k.n_vars + k.n_ineq + k.n_eq) for k in kids))},
        "roofline": {"bound": "hbm", "kernel": "k_batch_solve (persistent, whole PDHG loop per child)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "algorithmic_bytes": alg, "traffic": None},
        "clocks": clk.summary(),
    }
    if args.cpu_baseline:
        line["cpu_baseline"] = branching_cpu_baseline(kids, lp.objective, args.cpu_budget)
    return line


BRANCH_WORKLOAD = ("strong branching: the 40 child LPs of the 20 most fractional variables of a "
                   "set-covering node, m=200, n=2000 (seed 0)")


def cpu_baseline(p, args, ref_key=None):
    s = reference_sample(p, args.cpu_budget)
    ref_iters = load_reference_iterations(ref_key or args.config)
    out = {"unit": "solves/s", "cores": s["threads"], "kind": "port",
           "s_per_iter": s["s_per_iter"],
           "sample": (f"{s['iters']} iterations of the reference algorithm (C+OpenMP restatement of "
                      f"solver/lp/pdhg.py) on the standard form of the same LP, {s['seconds']:.1f} s; "
                      f"standard-form build {s['std_form_s']:.1f} s not included")}
    if ref_iters:
        n_it = ref_iters["iterations"]
        out["value"] = 1.0 / (s["s_per_iter"] * n_it)
        out["extrapolated_to_iters"] = n_it
        out["reference_status_at_that_count"] = ref_iters["status"]
    else:
        out["value"] = None
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return None
    if args.config == 3:
        return run_reference_batch(args, world)
    if args.config == 5:
        return run_reference_branching(args, world)
    if args.config == 4:
        from sovereign_solver_gb300.workloads import TransportFamily
        p = TransportFamily().problem(TEST_SEED0)
        cfg = {"workload": warmstart_workload(args.batch or 1000)}
        ref_key = f"4:{TEST_SEED0}"
    else:
        p, info, cfg = make_workload(args.config, seed=args.seed, powerlaw_nnz=args.powerlaw_nnz)
        ref_key = args.config
    for _ in range(args.warmup):
        reference_sample(p, min(2.0, args.cpu_budget))
    spi = []
    for _ in range(args.steps):
        s = reference_sample(p, args.cpu_budget)
        spi.append(s["s_per_iter"])
    ref_iters = load_reference_iterations(ref_key)
    n_it = ref_iters["iterations"] if ref_iters else None
    s_per_iter = statistics.median(spi)
    value = 1.0 / (s_per_iter * n_it) if n_it else None
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": s_per_iter * n_it * 1e3 if n_it else None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic", "config": {**cfg, "tol_rel_kkt": args.tol},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": s["threads"], "kind": "port",
                         "sample": (f"per step {s['iters']} iterations of the reference algorithm (C+OpenMP "
                                    f"restatement of solver/lp/pdhg.py), extrapolated to the "
                                    f"{n_it} iterations the reference needs on this LP "
                                    f"({ref_iters['status'] if ref_iters else 'unknown'})")},
        "s_per_iter": s_per_iter,
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if args.config in (0, 1) and args.ref_gpu:
        try:
            line["reference_gpu_path"] = reference_gpu_path(p)
        except Exception as exc:       # a secondary figure: its failure is reported, not fatal
            line["reference_gpu_path"] = {"unavailable": f"{type(exc).__name__}: {exc}"}
    if ref_iters:
        line["reference_run"] = {
            "value_is": ("rate of producing the reference's own answer on this LP: the timed per-iteration "
                         "cost x the iteration count of a full reference run made once in the build "
                         "container (tests/golden/reference_iterations.json)"),
            "iterations": n_it, "status": ref_iters["status"], "objective": ref_iters.get("objective"),
            "reaches_tol": ref_iters["status"] == "optimal"}
    return line


def run_reference_batch(args, world):
    """Reference arm of the batched workload: the reference algorithm on the
    32-LP sample, one single-threaded process per host core, once per step."""
    vals = []
    for _ in range(max(1, args.warmup // 3)):
        batch_cpu_baseline(args)
    for _ in range(args.steps):
        vals.append(batch_cpu_baseline(args))
    value = statistics.median(v["value"] for v in vals)
    cb = dict(vals[-1])
    cb["value"] = value
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic", "config": {"workload": batch_workload(args.batch or 4096), "tol_rel_kkt": args.tol},
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def run_reference_branching(args, world):
    """Reference arm of the strong-branching workload: one simplex solve per
    child (the reference's _lp_gain loop) on a budgeted sample per step."""
    _, lp, top, kids = branching_node(args, 0, on_cpu=True)
    for _ in range(max(1, args.warmup // 3)):
        branching_cpu_baseline(kids[:1], lp.objective, 0.0)
    vals = [branching_cpu_baseline(kids, lp.objective, args.cpu_budget) for _ in range(args.steps)]
    value = statistics.median(v["value"] for v in vals)
    cb = dict(vals[-1])
    cb["value"] = value
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "child LPs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic", "config": {"workload": BRANCH_WORKLOAD, "tol_rel_kkt": args.tol},
        "solver_tolerance": "exact (simplex, one solve per child as the reference's _lp_gain)",
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "child LPs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


# --------------------------------------------------------------------------- distributed plumbing
def instance_range(rank: int, per_rank: int, first: int = 0):
    """Instances of rank r (weak scaling: every rank its own disjoint block)."""
    return first + rank * per_rank, first + (rank + 1) * per_rank


def job_throughput(gathered, units_key: str, time_key: str, steps: int, time_scale: float = 1.0):
    """Whole-job rate: all ranks' units per step / the slowest rank's time per step.
    Returns (units per second, slowest rank's total time in seconds)."""
    t_max = max(g[time_key] for g in gathered) * time_scale
    total = sum(g[units_key] for g in gathered)
    return total * steps / t_max, t_max


def init_dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def gather(world, obj):
    if world == 1:
        return [obj]
    import torch.distributed as dist
    out = [None] * world
    dist.all_gather_object(out, obj)
    return out


def torchrun_command(argv, gpus: int, port: int):
    """The command that relaunches this script as ``gpus`` ranks of one node
    (one process per GPU, rendezvous on 127.0.0.1)."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
            "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__), *argv]


def free_port() -> int:
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


SUBRECORDS = (("planted_200x500", 0), ("powerlaw_1Mx2M", 2), ("batched_4096", 3), ("learned_warm_start_1000", 4))


def subrecords(args, rank, world):
    """The metric's other parts, measured in the same run as the default line:
    the planted 200x500 LP (time and attempts to tolerance), the power-law LP (SpMV roofline of both passes), the 4096-LP batch (solves/s,
    p50/p99 attempts) and the learned warm start (warm batched against cold
    single-instance wall time per solve).  Each has its own steps, clocks,
    roofline and CPU baseline; fewer timed steps than the default line, since
    one step of these is a whole batch or a multi-second solve."""
    import copy
    out = {}
    for name, cfg in SUBRECORDS:
        sub = copy.copy(args)
        sub.config, sub.steps, sub.warmup = cfg, args.sub_steps, args.sub_warmup
        if cfg == 0:                      # a few-ms solve: enough steps for a stable mean
            sub.steps = max(args.sub_steps, 20)
        sub.e2e_steps = 1
        sub.cpu_budget = min(args.cpu_budget, 10.0)
        sub.batch = {3: 4096, 4: 1000}.get(cfg)
        try:
            line = RUNNERS[cfg](sub, rank, world)
            line.pop("metric", None)
            out[name] = line
        except Exception as exc:          # a failed part is reported, the default line still prints
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
        log(f"subrecord {name}: {json.dumps(out[name])[:300]}")
    return out


RUNNERS = {0: run_ours, 1: run_ours, 2: run_ours, 3: run_batch, 4: run_warmstart, 5: run_branching}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1,
                    help="0: planted 200x500; 1: transportation 1000x2000 (default); 2: power-law 1Mx2M; "
                         "3: batched planted LPs (--batch of them); 4: learned warm start on the "
                         "transportation family (--batch held-out seeds); 5: strong branching "
                         "(40 child LPs of a set-covering MILP node in one batch)")
    ap.add_argument("--batch", type=int, default=None,
                    help="instances per GPU: config 3 default 4096, config 4 default 1000")
    ap.add_argument("--powerlaw-nnz", type=int, default=20_000_000,
                    help="config 2: nonzeros the Zipf(1.5) row lengths are rescaled to; 0 = lengths as drawn "
                         "(about 1.1e8 nonzeros)")
    ap.add_argument("--kkt-form", default="auto", choices=["auto", "lagrangian", "pdlp"],
                    help="single-LP error form the solve terminates on: auto = pdlp for config 2, else lagrangian")
    ap.add_argument("--single-sample", type=int, default=32)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--tol", type=float, default=TOL)
    ap.add_argument("--max-iters", type=int, default=100000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-ref-gpu", dest="ref_gpu", action="store_false",
                    help="reference arm: skip timing the reference's own torch-CUDA path from baseline/_ref")
    ap.add_argument("--no-subrecords", dest="subrecords", action="store_false",
                    help="default workload only: skip the power-law, batched and warm-start parts")
    ap.add_argument("--sub-steps", type=int, default=1, help="timed steps of each part of the default run")
    ap.add_argument("--sub-warmup", type=int, default=3, help="warm-up steps of each part of the default run")
    ap.add_argument("--graph-mode", type=int, default=2,
                    help="2: one graph with a device-driven loop (default); 1: replayed window graph; "
                         "0: plain launches (what a profiler's launch list can see kernel by kernel)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch under torch.distributed.run
        cmd = torchrun_command(sys.argv[1:], args.gpus, free_port())
        raise SystemExit(subprocess.call(cmd))
    rank, world = init_dist()
    args.device = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        if args.config == 3:
            args.batch = args.batch or 4096
        elif args.config == 4:
            args.batch = args.batch or 1000
        line = RUNNERS[args.config](args, rank, world)
        if args.subrecords and args.config == 1 and world == 1 and line is not None:
            line["subrecords"] = subrecords(args, rank, world)
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
