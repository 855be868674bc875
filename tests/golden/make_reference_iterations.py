"""Record how many iterations the reference algorithm needs on each benchmark
workload, and what it returns at its default iteration cap.

Runs the oracle's C + OpenMP restatement of ``solver/lp/pdhg.py`` (iteration-
exact with the reference on every golden vector) to a relative KKT tolerance of
1e-4 with the reference's default cap ``MAX_PDHG_ITERS = 100000``
(``solver/config.py:37``).  ``bench.py`` turns a timed sample of iterations into
the reference's time per solve with these counts.

    python tests/golden/make_reference_iterations.py      # writes reference_iterations.json
    python tests/golden/make_reference_iterations.py 3    # only the batched workload's sample
"""

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import sovereign_solver_gb300.workloads as wl  # noqa: E402
from oracle import pdhg_ref_c  # noqa: E402

CASES = {
    "0": lambda: wl.planted_lp(seed=0)[0],
    "1": lambda: wl.transportation_lp(1000, 2000, seed=0)[0],
}
# batched workload: every 128th instance of the 4096 (32 instances)
for _k in range(0, 4096, 128):
    CASES[f"3:{_k}"] = (lambda k: lambda: wl.batch_planted_lp(k)[0])(_k)
# learned warm start: the first 8 held-out seeds of the transportation family
_FAM = []
for _s in range(8):
    CASES[f"4:{10_000_000 + _s}"] = (lambda s: lambda: (_FAM or _FAM.append(wl.TransportFamily()) or _FAM)[0].problem(s))(
        10_000_000 + _s)


def main():
    out = {}
    path = os.path.join(HERE, "reference_iterations.json")
    keys = sys.argv[1:] or sorted(CASES)
    if keys == ["3"] or keys == ["4"]:
        keys = sorted(k for k in CASES if k.startswith(keys[0] + ":"))
    for key in keys:
        p = CASES[key]()
        t0 = time.perf_counter()
        r = pdhg_ref_c.solve(p, max_iters=100000, tol=1e-4)
        dt = time.perf_counter() - t0
        out[key] = {"iterations": r.iterations, "status": r.status, "tol": 1e-4, "max_iters": 100000,
                    "objective": r.objective, "seconds": round(dt, 1), "threads": pdhg_ref_c.threads(),
                    "workload": p.name}
        print(key, out[key], flush=True)
    old = {}
    if os.path.exists(path):
        with open(path) as f:
            old = json.load(f)
    old.update(out)
    with open(path, "w") as f:
        json.dump(old, f, indent=1)


if __name__ == "__main__":
    main()
