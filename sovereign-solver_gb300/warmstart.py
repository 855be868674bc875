"""Learned warm start for a parametric LP family: data, training, evaluation.

Pipeline (every step on the GPU through this package):
  1. ``solve_family`` solves the training seeds cold with the batched solver
     (tolerance 1e-4) and keeps each solution (x sparse, y, the final primal
     weight) plus the instance's scaled costs (FP16) and right-hand sides;
  2. ``train`` fits ``WarmStartGNN`` on them with its own forward / backward /
     Adam kernels (minibatches of ``net.max_batch`` instances);
  3. ``evaluate`` compares, on held-out seeds, cold single-instance PDHG with the
     learned-warm-start batched PDHG (GNN inference included), both judged by
     the engine's relative-KKT test.

Run as a script to train on the transportation family and save the weights:
    python sovereign-solver_gb300/warmstart.py --train 20000 --test 1000 --out weights.npz
"""

from __future__ import annotations

import os
import sys
import time
from dataclasses import dataclass, field

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import sovereign_solver_gb300 as _pkg  # noqa: F401
    __package__ = "sovereign_solver_gb300"

from .batch import PDHGBatch
from .gnn import WarmStartGNN
from .pdhg import PDHGEngine
from .problem import Problem
from .workloads import TransportFamily


def family_instance(template: Problem, c, b_ub, b_eq, name: str = "") -> Problem:
    """An instance of ``template``'s family: same matrices and bounds, new c and b."""
    return Problem(c=np.asarray(c, float), A_ub=template.A_ub, b_ub=np.asarray(b_ub, float), A_eq=template.A_eq,
                   b_eq=np.asarray(b_eq, float), lb=template.lb, ub=template.ub,
                   integer_mask=template.integer_mask, name=name)


def transport_instances(fam: TransportFamily, template: Problem, seeds):
    out = []
    for s in seeds:
        cost, supply, demand = fam.params(int(s))
        out.append(family_instance(template, cost, supply, demand, f"transport_{fam.S}x{fam.D}_s{s}"))
    return out


@dataclass
class FamilyData:
    seeds: np.ndarray
    c: np.ndarray                   # (k, n) FP16: c / c_scale
    b: np.ndarray                   # (k, m) FP32: b / b_scale
    x_ptr: np.ndarray               # sparse x* (CSR over instances)
    x_idx: np.ndarray
    x_val: np.ndarray               # FP32, original units
    y: np.ndarray                   # (k, m) FP32
    omega: np.ndarray               # (k,) final primal weight (engine scale)
    iterations: np.ndarray
    optimal: np.ndarray
    solve_s: float = 0.0
    extra: dict = field(default_factory=dict)

    def x_dense(self, i: int, n: int) -> np.ndarray:
        x = np.zeros(n, np.float32)
        a, b = self.x_ptr[i], self.x_ptr[i + 1]
        x[self.x_idx[a:b]] = self.x_val[a:b]
        return x


def solve_family(net: WarmStartGNN, fam: TransportFamily, template: Problem, seeds, tol: float = 1e-4,
                 chunk: int = 1024, device: int = 0, log=print) -> FamilyData:
    """Cold batched solves of ``seeds``; solutions and features for training."""
    seeds = np.asarray(seeds)
    k, n, m = len(seeds), net.n, net.m
    cs = np.empty((k, n), np.float16)
    bs = np.empty((k, m), np.float32)
    y = np.empty((k, m), np.float32)
    omega = np.empty(k)
    its = np.empty(k, np.int64)
    opt = np.empty(k, bool)
    xp, xi, xv = [0], [], []
    thresh = 1e-7 * net.scales["x"]
    t_solve = 0.0
    for s0 in range(0, k, chunk):
        sl = seeds[s0:s0 + chunk]
        probs = transport_instances(fam, template, sl)
        t = time.perf_counter()
        with PDHGBatch(probs, tol=tol, device=device) as b:
            res = b.solve()
        t_solve += time.perf_counter() - t
        for q, (p, r) in enumerate(zip(probs, res)):
            i = s0 + q
            cs[i] = p.c / net.scales["c"]
            bs[i] = np.concatenate([p.b_ub, p.b_eq]) / net.scales["b"]
            y[i] = r.y
            omega[i] = r.stats["primal_weight"]
            its[i] = r.iterations
            opt[i] = r.status == "optimal"
            nz = np.flatnonzero(r.x > thresh)
            xi.append(nz.astype(np.int32))
            xv.append(r.x[nz].astype(np.float32))
            xp.append(xp[-1] + nz.size)
        if log:
            log(f"solved {min(k, s0 + chunk)}/{k} seeds ({t_solve:.1f}s in solves; "
                f"median {np.median(its[:s0 + len(sl)]):.0f} iterations)")
    return FamilyData(seeds, cs, bs, np.asarray(xp, np.int64), np.concatenate(xi) if xi else np.zeros(0, np.int32),
                      np.concatenate(xv) if xv else np.zeros(0, np.float32), y, omega, its, opt, t_solve)


def _batch_arrays(net: WarmStartGNN, data: FamilyData, rows):
    fvs, fcs, xts, yts, lts = [], [], [], [], []
    for i in rows:
        fv, fc = net.features_from(data.c[i].astype(float) * net.scales["c"], data.b[i].astype(float) * net.scales["b"])
        xt, yt, lt = net.targets(data.x_dense(i, net.n), data.y[i], data.omega[i])
        fvs.append(fv); fcs.append(fc); xts.append(xt); yts.append(yt); lts.append(lt)
    return fvs, fcs, xts, yts, np.asarray(lts, np.float32)


def train(net: WarmStartGNN, data: FamilyData, epochs: int = 5, seed: int = 0, log=print) -> list:
    """Minibatch training over the optimal instances of ``data``; returns the mean loss per epoch."""
    rng = np.random.default_rng(seed)
    rows = np.flatnonzero(data.optimal)
    hist = []
    for ep in range(epochs):
        rng.shuffle(rows)
        t = time.perf_counter()
        tot, cnt = 0.0, 0
        for s in range(0, len(rows) - net.max_batch + 1, net.max_batch):
            tot += net.train_step(*_batch_arrays(net, data, rows[s:s + net.max_batch]))
            cnt += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {hist[-1]:.5f} ({time.perf_counter() - t:.1f}s)")
    return hist


def evaluate(net: WarmStartGNN, fam: TransportFamily, template: Problem, seeds, tol: float = 1e-4,
             single_sample: int = 32, device: int = 0) -> dict:
    """Warm (GNN + batched PDHG) versus cold (batched, and single-instance) on held-out seeds."""
    probs = transport_instances(fam, template, seeds)
    # cold single-instance PDHG, one LP at a time (create + solve + read-back per LP)
    single = []
    for p in probs[:single_sample]:
        t = time.perf_counter()
        with PDHGEngine(p, tol=tol, device=device) as eng:
            r = eng.solve()
        single.append((time.perf_counter() - t, r.iterations, r.status == "optimal"))
    # cold batched
    t = time.perf_counter()
    with PDHGBatch(probs, tol=tol, device=device) as b:
        cold = b.solve()
    t_cold = time.perf_counter() - t
    # learned warm start: inference + batched PDHG from the predictions (fallback on)
    t = time.perf_counter()
    starts = net.predict(probs)
    t_inf = time.perf_counter() - t
    with PDHGBatch(probs, tol=tol, device=device) as b:
        b.set_warm_starts(starts)
        warm = b.solve()
    t_warm = time.perf_counter() - t
    ci = np.array([r.iterations for r in cold])
    wi = np.array([r.iterations for r in warm])
    return {
        "count": len(probs),
        "cold_batched_iters_median": float(np.median(ci)), "warm_batched_iters_median": float(np.median(wi)),
        "cold_batched_iters_mean": float(ci.mean()), "warm_batched_iters_mean": float(wi.mean()),
        "iters_ratio_warm_over_cold": float(wi.mean() / ci.mean()),
        "warm_used": int(sum(r.stats["warm_start_used"] for r in warm)),
        "cold_optimal": int(sum(r.status == "optimal" for r in cold)),
        "warm_optimal": int(sum(r.status == "optimal" for r in warm)),
        "cold_batched_s_per_solve": t_cold / len(probs), "warm_batched_s_per_solve": t_warm / len(probs),
        "gnn_inference_s_per_instance": t_inf / len(probs),
        "cold_single_s_per_solve": float(np.mean([s[0] for s in single])),
        "cold_single_iters_median": float(np.median([s[1] for s in single])),
        "cold_single_optimal": int(sum(s[2] for s in single)), "single_sample": len(single),
        "warm_results": warm, "cold_results": cold, "problems": probs,
    }


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="train the learned warm start on the 200 x 400 transportation family")
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--test", type=int, default=1000)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default="warmstart_transport_200x400.npz")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    fam = TransportFamily()
    template = fam.problem(0)
    net = WarmStartGNN(template, max_batch=a.batch, lr=a.lr, device=a.device)
    data = solve_family(net, fam, template, np.arange(a.train), device=a.device)
    train(net, data, epochs=a.epochs)
    net.save(a.out)
    ev = evaluate(net, fam, template, np.arange(10_000_000, 10_000_000 + a.test), device=a.device)
    print({k: v for k, v in ev.items() if not isinstance(v, list)})


if __name__ == "__main__":
    main()
