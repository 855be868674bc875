"""Exact optima of the workloads with no planted optimum, for objective errors.

The transportation LPs (1000 x 2000, seed 0; the 200 x 400 family's first
held-out seed) have no planted solution.  Their optima come from HiGHS's dual
simplex as bundled in SciPy (``scipy.optimize.linprog(method="highs-ds")``,
SciPy 1.18.1), an exact vertex solver independent of this repository, run here
once; the values are committed to ``optima.json``.  Usage:

    python tests/golden/make_optima.py
"""

import json
import os
import sys
import time

import numpy as np
import scipy
from scipy.optimize import linprog

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import sovereign_solver_gb300.workloads as wl  # noqa: E402

HELD_OUT_SEED = 10_000_000      # first held-out seed of the learned warm start's test set


def highs(p):
    t = time.perf_counter()
    bounds = np.column_stack([p.lb, np.where(np.isinf(p.ub), None, p.ub)])
    r = linprog(p.c, A_ub=p.A_ub if p.n_ineq else None, b_ub=p.b_ub if p.n_ineq else None,
                A_eq=p.A_eq if p.n_eq else None, b_eq=p.b_eq if p.n_eq else None,
                bounds=bounds, method="highs-ds")
    if r.status != 0:
        raise RuntimeError(r.message)
    return {"objective": repr(float(r.fun)), "solver": f"scipy {scipy.__version__} linprog highs-ds",
            "seconds": round(time.perf_counter() - t, 1), "simplex_iterations": int(r.nit)}


def main():
    out = {}
    p, _ = wl.transportation_lp(1000, 2000, seed=0)
    out["transport_1000x2000_s0"] = highs(p)
    print("transport 1000x2000", out["transport_1000x2000_s0"], flush=True)
    p = wl.TransportFamily().problem(HELD_OUT_SEED)
    out[f"transport_family_200x400_s{HELD_OUT_SEED}"] = highs(p)
    print("family", out[f"transport_family_200x400_s{HELD_OUT_SEED}"], flush=True)
    with open(os.path.join(HERE, "optima.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
