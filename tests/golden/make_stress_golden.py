"""Generate the stress-LP golden fixtures by running the REFERENCE itself.

The reference benchmark runner builds three seeded "stress" LPs
(``benchmarks/run_benchmarks.py:314-378``: random_n50_m30, sparse_n500_m250,
badly_scaled_1e8) and publishes its PDHG results on them
(``benchmarks/results/benchmark_comparison.csv:27,31,35``).  This script calls
that builder unchanged: HiGHS (``highspy``, not installed here) is replaced by
an empty module and the runner's solver calls by stubs that only record the
problems, so the instances are the reference's own.  It then runs the
reference ``solve_lp_pdhg`` with the runner's settings (its defaults:
max_iters 100000, tol 1e-6) and reads the published rows from the CSV.  A
fourth LP comes the same way from the reference's own PDHG test
``test_pdhg_large_sparse_terminates`` (``tests/test_pdhg.py:137-156``, solver
call stubbed): it is unbounded, and the reference runs it to its cap.

Run from the repository root, in a container where the reference checkout is
mounted (pure Python, NumPy + SciPy):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_stress_golden.py <reference checkout>

(or with the checkout's path in SPS_REFERENCE_ROOT and no argument).

Writes ``stress_problems.npz`` (CSR arrays, the layout of
``small_problems.npz``) and ``stress_golden.json`` (reference result and the
published CSV row per problem, with the HiGHS optimum the CSV lists beside it).
"""

from __future__ import annotations

import csv
import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import pack  # noqa: E402


class _Skipped:
    status, objective, iterations = "skipped", 0.0, 0


def main(ref_root: str) -> None:
    sys.path.insert(0, ref_root)
    sys.modules.setdefault("highspy", types.ModuleType("highspy"))
    import benchmarks.run_benchmarks as rb
    from solver.lp.pdhg import solve_lp_pdhg

    problems = []

    def record(p, *args, **kw):
        problems.append(p)
        return _Skipped()

    rb.get_highs_lp_solution = lambda p, *a, **k: (0.0, 0.0, "")
    rb.solve_lp_revised = record                       # the first solver call per problem
    rb.solve_lp_ipm = lambda p, *a, **k: _Skipped()
    rb.solve_lp_pdhg = lambda p, *a, **k: _Skipped()
    rb.run_synthetic_stress_benchmarks([])

    # the reference's own PDHG test LP "large sparse" (tests/test_pdhg.py:137-156),
    # taken from that test function with its solver call stubbed
    import tests.test_pdhg as tp

    def record_test(p, *a, **k):
        p.name = "ref_test_large_sparse"
        problems.append(p)
        return types.SimpleNamespace(status="iteration_limit", x=np.zeros(p.n_vars))

    tp.solve_lp_pdhg = record_test
    tp.test_pdhg_large_sparse_terminates()

    published = {}
    with open(os.path.join(ref_root, "benchmarks", "results", "benchmark_comparison.csv")) as f:
        for row in csv.DictReader(f):
            if row["solver"] == "Sovereign PDHG":
                published[row["problem"]] = {"status": row["status"], "objective": row["objective"],
                                             "iterations": int(row["iters_nodes"]),
                                             "highs_objective": row["highs_obj"]}

    out, gold = {}, {}
    for p in problems:
        pack(p.name, p, out)
        t0 = time.perf_counter()
        r = solve_lp_pdhg(p)
        dt = time.perf_counter() - t0
        gold[p.name] = {"max_iters": 100000, "tol": 1e-6, "status": r.status,
                        "objective": repr(float(r.objective)), "iterations": int(r.iterations),
                        "ref_seconds": round(dt, 4), "published": published.get(p.name)}
        print(f"{p.name:18s} {r.status:16s} obj={r.objective!r} iters={r.iterations} ({dt:.2f}s); "
              f"published {published.get(p.name)}")
    np.savez_compressed(os.path.join(HERE, "stress_problems.npz"), **out)
    with open(os.path.join(HERE, "stress_golden.json"), "w") as f:
        json.dump(gold, f, indent=1)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPS_REFERENCE_ROOT")
    if not root:
        raise SystemExit(f"usage: python {sys.argv[0]} <reference checkout> (or set SPS_REFERENCE_ROOT)")
    main(root)
