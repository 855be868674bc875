"""Generate the golden fixtures in this folder by running the REFERENCE itself.

Run from the repository root, in a container where the reference checkout is
mounted (it is pure Python and imports with NumPy + SciPy):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <reference checkout>

(or with the checkout's path in SPS_REFERENCE_ROOT and no argument).

Writes
------
``netlib_problems.npz``   afiro, blending, adlittle, brandy read by the
                          reference's MPS reader (``solver/io/mps_reader.py:42``),
                          stored as CSR arrays so no MPS parser is needed later.
``small_problems.npz``    the reference test LPs (``tests/test_pdhg.py:37-170``,
                          ``tests/test_advanced.py:110-130``), a mixed-bounds LP
                          that exercises every branch of the standard-form
                          conversion, and the m=200 × n=500 planted LP (seeds 0-2).
``pdhg_golden.json``      for each problem: the reference ``solve_lp_pdhg``
                          result (status, objective as a repr'd float,
                          iterations) at the settings named in the entry,
                          plus the reference revised-simplex objective.
``stdform_golden.npz``    the reference ``_to_standard_form_pdhg`` and
                          ``_compute_step_sizes`` outputs for the mixed-bounds LP.
"""

from __future__ import annotations

import json
import os
import sys
import time

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def pack(prefix, p, out):
    out[f"{prefix}/c"] = np.asarray(p.c, float)
    for nm in ("A_ub", "A_eq"):
        M = sp.csr_matrix(p.__getattribute__(nm), dtype=float)
        out[f"{prefix}/{nm}/data"] = M.data
        out[f"{prefix}/{nm}/indices"] = M.indices.astype(np.int32)
        out[f"{prefix}/{nm}/indptr"] = M.indptr.astype(np.int32)
        out[f"{prefix}/{nm}/shape"] = np.array(M.shape, np.int64)
    out[f"{prefix}/b_ub"] = np.asarray(p.b_ub, float)
    out[f"{prefix}/b_eq"] = np.asarray(p.b_eq, float)
    out[f"{prefix}/lb"] = np.asarray(p.lb, float)
    out[f"{prefix}/ub"] = np.asarray(p.ub, float)
    out[f"{prefix}/sense"] = np.array(p.sense)


def make_lp(RefProblem, c, A_ub, b_ub, A_eq=None, b_eq=None, lb=None, ub=None):
    n = len(c)
    A_ub = np.asarray(A_ub, float).reshape(-1, n)
    if A_eq is None:
        A_eq, b_eq = np.zeros((0, n)), np.zeros(0)
    return RefProblem(
        c=np.asarray(c, float), A_ub=sp.csr_matrix(A_ub), b_ub=np.asarray(b_ub, float),
        A_eq=sp.csr_matrix(np.asarray(A_eq, float).reshape(-1, n)), b_eq=np.asarray(b_eq, float),
        lb=np.zeros(n) if lb is None else np.asarray(lb, float),
        ub=np.full(n, np.inf) if ub is None else np.asarray(ub, float),
        integer_mask=np.zeros(n, dtype=bool))


def main(ref_root: str) -> None:
    sys.path.insert(0, ref_root)
    sys.path.insert(0, REPO)
    from solver.problem import Problem as RefProblem
    from solver.io.mps_reader import read_mps
    from solver.lp.pdhg import solve_lp_pdhg, _to_standard_form_pdhg, _compute_step_sizes
    from solver.lp.simplex_revised import solve_lp_revised
    import sovereign_solver_gb300.workloads as wl

    problems = {}
    settings = {}
    for nm in ("afiro", "blending", "adlittle", "brandy"):
        problems[nm] = read_mps(os.path.join(ref_root, "benchmarks", "instances", nm + ".mps"))
        settings[nm] = {"max_iters": 25000, "tol": 1e-6}   # benchmarks/run_benchmarks.py:221

    # reference unit-test LPs (default max_iters / tol)
    problems["t_2var"] = make_lp(RefProblem, [-3.0, -5.0], [[1, 0], [0, 2], [3, 2]], [4, 12, 18])
    problems["t_simple_min"] = make_lp(RefProblem, [1.0, 2.0], [[-1.0, -1.0]], [-2.0])
    problems["t_trivial"] = make_lp(RefProblem, [1, 1], [[1, 0], [0, 1]], [3, 3])
    problems["t_xplus2y"] = make_lp(RefProblem, [-1, -2], [[1, 1]], [4])
    rng = np.random.default_rng(42)
    A = np.abs(rng.standard_normal((4, 6)))
    xt = rng.uniform(0.5, 1.5, 6)
    b = A @ xt + rng.uniform(0.1, 0.5, 4)
    cr = rng.standard_normal(6)
    problems["t_random46"] = make_lp(RefProblem, cr, np.vstack([A, np.eye(6)]),
                                     np.concatenate([b, np.full(6, 3.0)]))
    problems["t_ub_simple"] = make_lp(RefProblem, [1.0], [[1.0]], [3.0], lb=[0.0], ub=[2.0])
    problems["t_ub_tight"] = make_lp(RefProblem, [-1.0], [[1.0]], [10.0], lb=[0.0], ub=[5.0])
    for k in problems:
        settings.setdefault(k, {"max_iters": 100000, "tol": 1e-6})

    # mixed bounds: finite/infinite lb and ub, negative rhs, equality rows, a max problem
    rng = np.random.default_rng(2024)
    n, mu, me = 12, 5, 3
    Aub = rng.standard_normal((mu, n)) * (rng.random((mu, n)) < 0.6)
    Aeq = rng.standard_normal((me, n)) * (rng.random((me, n)) < 0.6)
    x0 = rng.uniform(0.2, 1.0, n)
    lb = np.where(rng.random(n) < 0.7, rng.uniform(-1.0, 0.1, n), -np.inf)
    ub = np.where(rng.random(n) < 0.5, x0 + rng.uniform(0.5, 2.0, n), np.inf)
    bub = Aub @ x0 + rng.uniform(0.0, 0.5, mu) - 1.5
    beq = Aeq @ x0
    mixed = make_lp(RefProblem, rng.uniform(0.5, 2.0, n), Aub, bub, Aeq, beq, lb, ub)
    mixed.sense = "max"
    mixed.c = -mixed.c
    problems["mixed_bounds"] = mixed
    settings["mixed_bounds"] = {"max_iters": 20000, "tol": 1e-6}

    for s in range(3):
        p, info = wl.planted_lp(seed=s)
        problems[f"planted200x500_s{s}"] = p
        settings[f"planted200x500_s{s}"] = {"max_iters": 100000, "tol": 1e-4,
                                            "obj_star": info["obj_star"]}

    out = {}
    for k, p in problems.items():
        pack(k, p, out)
    netlib = {k: v for k, v in out.items() if k.split("/")[0] in
              ("afiro", "blending", "adlittle", "brandy")}
    small = {k: v for k, v in out.items() if k not in netlib}
    np.savez_compressed(os.path.join(HERE, "netlib_problems.npz"), **netlib)
    np.savez_compressed(os.path.join(HERE, "small_problems.npz"), **small)

    gold = {}
    for k, p in problems.items():
        st = settings[k]
        t0 = time.perf_counter()
        r = solve_lp_pdhg(p, max_iters=st["max_iters"], tol=st["tol"])
        dt = time.perf_counter() - t0
        entry = {"max_iters": st["max_iters"], "tol": st["tol"], "status": r.status,
                 "objective": repr(float(r.objective)), "iterations": int(r.iterations),
                 "x": [repr(float(v)) for v in r.x] if r.x.size <= 64 else None,
                 "ref_seconds": round(dt, 4)}
        if "obj_star" in st:
            entry["obj_star"] = repr(float(st["obj_star"]))
        if k.startswith("planted"):
            entry["simplex_objective"] = None     # the reference simplex needs ~1 min here
        else:
            s = solve_lp_revised(p)
            entry["simplex_status"] = s.status
            entry["simplex_objective"] = repr(float(s.objective)) if s.status == "optimal" else None
        gold[k] = entry
        print(f"{k:22s} {r.status:16s} obj={r.objective!r} iters={r.iterations} ({dt:.2f}s)")
    with open(os.path.join(HERE, "pdhg_golden.json"), "w") as f:
        json.dump(gold, f, indent=1)

    c, A_std, b_std, lbf, n_orig = _to_standard_form_pdhg(mixed)
    tau, sigma = _compute_step_sizes(A_std)
    A_std = sp.csr_matrix(A_std)
    np.savez_compressed(os.path.join(HERE, "stdform_golden.npz"), c=c, A=A_std.toarray(),
                        b=b_std, lb_shift=lbf, n_orig=np.int64(n_orig), tau=tau, sigma=sigma)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPS_REFERENCE_ROOT")
    if not root:
        raise SystemExit(f"usage: python {sys.argv[0]} <reference checkout> (or set SPS_REFERENCE_ROOT)")
    main(root)
