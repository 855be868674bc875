"""Seeded synthetic LP generators for the five benchmark workloads.

Every generator is deterministic in its seed (``numpy.random.default_rng``)
and returns a :class:`Problem` plus an ``info`` dict.  Generators with a
planted optimum put ``x_star``, ``y_star`` and ``obj_star`` in ``info``.

Planted construction ("random feasible bounded LP"): draw A, pick x* ∈ [0,1]
on 60 % of the columns (0 elsewhere), y* ~ N(0,1), s* ~ Exp(1) only where
x* = 0; set b = A x*, c = Aᵀy* + s*, l = 0, u = U.  Then (x*, y*, s*) satisfies
the KKT conditions of ``min cᵀx, Ax = b, 0 ≤ x ≤ U`` (x* < U, s* ⊥ x*), so
x* is optimal with objective cᵀx* = bᵀy* exactly.

Workloads (sizes as named):

* ``planted_lp``            m=200, n=500, 5 % density equality LP, u = 2.
* ``transportation_lp``     S sources × D sinks; supply rows ≤, demand rows =;
                            costs are Euclidean distances of uniform points plus
                            U[0, 0.1]; Σ supply = 1.05 Σ demand.  Row layout
                            follows ``demos/transportation_lp.py:125-146``
                            (variable i·D + j ships source i → sink j).
* ``powerlaw_lp``           m=1M, n=2M, Zipf(1.5) row lengths clipped to
                            [2, 5000], planted, u = 10 (optionally rescaled to
                            a target nonzero count).
* ``batch_planted_lp``      instance k of the 4096-LP batch: m log-uniform in
                            [50, 5000], n = round(m·U[1.5, 3]), 10–50 nonzeros
                            per column, planted, u = 2.
* ``transport_family``      200 × 400 transportation LPs on one fixed
                            geometry; per-seed demand × U[0.8, 1.2] and cost
                            × (1 + N(0, 0.05)).
* ``set_cover_milp``        a node of a branch-and-bound search: 0/1 set
                            covering, m = 200 rows, n = 2000 binaries, 2 %
                            density (strong branching's parent problem).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from .problem import Problem


def _plant(A: sp.csr_matrix, rng: np.random.Generator, u: float):
    """Planted optimum on a given matrix: returns (b, c, x*, y*, obj*)."""
    m, n = A.shape
    support = rng.random(n) < 0.6
    x_star = np.where(support, rng.random(n), 0.0)
    y_star = rng.standard_normal(m)
    s_star = np.where(support, 0.0, rng.exponential(1.0, n))
    b = A @ x_star
    c = A.T @ y_star + s_star
    obj = float(b @ y_star)
    return b, c, x_star, y_star, obj


def _fill_empty_columns(rows: np.ndarray, cols: np.ndarray, m: int, n: int,
                        rng: np.random.Generator):
    """Give every column with no entry one entry in a uniformly random row."""
    present = np.zeros(n, dtype=bool)
    present[cols] = True
    empty = np.flatnonzero(~present)
    if empty.size:
        rows = np.concatenate([rows, rng.integers(0, m, empty.size)])
        cols = np.concatenate([cols, empty])
    return rows, cols


def _distinct_per_group(group_sizes: np.ndarray, universe: int,
                        rng: np.random.Generator, exact: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """For each group g draw group_sizes[g] distinct members of range(universe).

    Draw with replacement, drop duplicates inside each group, redraw the
    shortfall, repeat; exact "without replacement" semantics for any size
    ≤ universe.  With ``exact=False`` the duplicates are only dropped (for
    group sizes far below the universe, where they are rare).  Returns
    (group_id, member) pairs sorted by (group, member).
    """
    k = np.minimum(group_sizes.astype(np.int64), universe)
    groups = np.repeat(np.arange(k.size, dtype=np.int64), k)
    members = rng.integers(0, universe, groups.size)
    while True:
        key = groups * universe + members
        key.sort()
        key = key[np.concatenate(([True], key[1:] != key[:-1]))] if key.size else key
        if not exact:
            return key // universe, key % universe
        g = key // universe
        have = np.bincount(g, minlength=k.size)
        short = k - have
        if not short.any():
            return g, key % universe
        extra_g = np.repeat(np.arange(k.size, dtype=np.int64), short)
        groups = np.concatenate([g, extra_g])
        members = np.concatenate([key % universe, rng.integers(0, universe, extra_g.size)])


def planted_lp(m: int = 200, n: int = 500, density: float = 0.05, u: float = 2.0,
               seed: int = 0) -> tuple[Problem, dict]:
    """Random feasible bounded equality LP with a planted optimum (m=200, n=500 default)."""
    rng = np.random.default_rng(seed)
    mask = rng.random((m, n)) < density
    rows, cols = np.nonzero(mask)
    rows, cols = _fill_empty_columns(rows, cols, m, n, rng)
    vals = rng.standard_normal(rows.size)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(m, n))
    A.sum_duplicates()
    A.sort_indices()
    b, c, xs, ys, obj = _plant(A, rng, u)
    p = Problem(c=c, A_ub=sp.csr_matrix((0, n)), b_ub=np.zeros(0), A_eq=A, b_eq=b,
                lb=np.zeros(n), ub=np.full(n, u), integer_mask=np.zeros(n, dtype=bool),
                name=f"planted_{m}x{n}_s{seed}")
    return p, {"x_star": xs, "y_star": ys, "obj_star": obj}


def transportation_lp(n_src: int = 1000, n_dst: int = 2000, seed: int = 0,
                      ) -> tuple[Problem, dict]:
    """Unbalanced transportation LP (supply ≤, demand =), 1000 × 2000 default."""
    rng = np.random.default_rng(seed)
    P = rng.random((n_src, 2))
    Q = rng.random((n_dst, 2))
    supply = rng.uniform(50.0, 150.0, n_src)
    dem = rng.random(n_dst)
    dem *= supply.sum() / (1.05 * dem.sum())
    # cost built row by row to keep peak memory at one n-vector plus a row block
    cost = np.empty(n_src * n_dst)
    blk = max(1, (1 << 22) // n_dst)
    for s in range(0, n_src, blk):
        e = min(n_src, s + blk)
        d = np.sqrt(((P[s:e, None, :] - Q[None, :, :]) ** 2).sum(-1))
        cost[s * n_dst:e * n_dst] = (d + 0.1 * rng.random((e - s, n_dst))).ravel()
    return _transport_problem(cost, supply, dem, n_src, n_dst,
                              f"transport_{n_src}x{n_dst}_s{seed}"), {}


def _transport_problem(cost, supply, demand, S, D, name) -> Problem:
    n = S * D
    ones = np.ones(n)
    A_ub = sp.csr_matrix((ones, np.arange(n, dtype=np.int32),
                          np.arange(0, n + 1, D, dtype=np.int32)), shape=(S, n))
    eq_cols = (np.arange(D, dtype=np.int64)[:, None] + D * np.arange(S, dtype=np.int64)[None, :])
    A_eq = sp.csr_matrix((ones, eq_cols.ravel().astype(np.int32),
                          np.arange(0, n + 1, S, dtype=np.int32)), shape=(D, n))
    return Problem(c=cost, A_ub=A_ub, b_ub=np.asarray(supply, float), A_eq=A_eq,
                   b_eq=np.asarray(demand, float), lb=np.zeros(n), ub=np.full(n, np.inf),
                   integer_mask=np.zeros(n, dtype=bool), name=name)


def powerlaw_lp(m: int = 1_000_000, n: int = 2_000_000, target_nnz: int | None = 20_000_000,
                u: float = 10.0, seed: int = 0) -> tuple[Problem, dict]:
    """Power-law-row LP: Zipf(1.5) row lengths clipped to [2, 5000], planted, u = 10.

    With ``target_nnz=None`` the lengths are used as drawn (≈1.1e8 nonzeros at
    m=1M).  With a target, lengths are rescaled by target/Σlength (floor 2),
    which keeps the power-law shape at the stated nonzero count.  Columns in a
    row are distinct and uniform over range(n).
    """
    rng = np.random.default_rng(seed)
    L = np.clip(rng.zipf(1.5, m), 2, 5000).astype(np.int64)
    if target_nnz is not None:
        L = np.maximum(2, np.floor(L * (target_nnz / L.sum()))).astype(np.int64)
    # rows of at most 5000 distinct columns out of 2M: duplicate draws are rare
    # (≈ L²/2n per row) and are dropped rather than redrawn
    rows, cols = _distinct_per_group(L, n, rng, exact=False)
    present = np.zeros(n, dtype=bool)
    present[cols] = True
    empty = np.flatnonzero(~present)
    if empty.size:   # one entry in a random row for every empty column, merged in row order
        er = rng.integers(0, m, empty.size)
        key = np.concatenate([rows * n + cols, er * n + empty])
        key.sort()
        rows, cols = key // n, key % n
    vals = rng.standard_normal(rows.size)
    indptr = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=m), out=indptr[1:])
    A = sp.csr_matrix((vals, cols.astype(np.int32), indptr.astype(np.int32)), shape=(m, n))
    b, c, xs, ys, obj = _plant(A, rng, u)
    p = Problem(c=c, A_ub=sp.csr_matrix((0, n)), b_ub=np.zeros(0), A_eq=A, b_eq=b,
                lb=np.zeros(n), ub=np.full(n, u), integer_mask=np.zeros(n, dtype=bool),
                name=f"powerlaw_{m}x{n}_nnz{A.nnz}_s{seed}")
    return p, {"x_star": xs, "y_star": ys, "obj_star": obj}


def batch_planted_lp(k: int, m_range=(50, 5000), n_ratio=(1.5, 3.0), col_nnz=(10, 50),
                     u: float = 2.0) -> tuple[Problem, dict]:
    """Instance k of the batched workload (seed k)."""
    rng = np.random.default_rng(k)
    m = int(round(np.exp(rng.uniform(np.log(m_range[0]), np.log(m_range[1])))))
    n = int(round(m * rng.uniform(*n_ratio)))
    per_col = np.minimum(rng.integers(col_nnz[0], col_nnz[1] + 1, n), m)
    cols, rows = _distinct_per_group(per_col, m, rng)
    vals = rng.standard_normal(rows.size)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(m, n))
    A.sort_indices()
    b, c, xs, ys, obj = _plant(A, rng, u)
    p = Problem(c=c, A_ub=sp.csr_matrix((0, n)), b_ub=np.zeros(0), A_eq=A, b_eq=b,
                lb=np.zeros(n), ub=np.full(n, u), integer_mask=np.zeros(n, dtype=bool),
                name=f"batch_{k}_{m}x{n}")
    return p, {"x_star": xs, "y_star": ys, "obj_star": obj}


class TransportFamily:
    """Parametric 200 × 400 transportation family on one fixed geometry.

    The geometry (points, base costs, base supplies, base demands) comes from
    ``family_seed``; instance ``seed`` perturbs demand × U[0.8, 1.2] and cost
    × (1 + N(0, 0.05)), then rescales supply so Σ supply = 1.05 Σ demand.
    """

    def __init__(self, n_src: int = 200, n_dst: int = 400, family_seed: int = 12345):
        rng = np.random.default_rng(family_seed)
        self.S, self.D = n_src, n_dst
        P = rng.random((n_src, 2))
        Q = rng.random((n_dst, 2))
        d = np.sqrt(((P[:, None, :] - Q[None, :, :]) ** 2).sum(-1))
        self.base_cost = (d + 0.1 * rng.random((n_src, n_dst))).ravel()
        self.base_supply = rng.uniform(50.0, 150.0, n_src)
        dem = rng.random(n_dst)
        self.base_demand = dem * self.base_supply.sum() / (1.05 * dem.sum())

    def params(self, seed: int):
        """(cost, supply, demand) of instance ``seed``."""
        rng = np.random.default_rng(1_000_003 * (seed + 1))
        demand = self.base_demand * rng.uniform(0.8, 1.2, self.D)
        cost = self.base_cost * (1.0 + 0.05 * rng.standard_normal(self.base_cost.size))
        supply = self.base_supply * (1.05 * demand.sum() / self.base_supply.sum())
        return cost, supply, demand

    def problem(self, seed: int) -> Problem:
        cost, supply, demand = self.params(seed)
        return _transport_problem(cost, supply, demand, self.S, self.D,
                                  f"transport_family_{self.S}x{self.D}_s{seed}")


def transport_family(seed: int, family: TransportFamily | None = None) -> tuple[Problem, dict]:
    fam = family or TransportFamily()
    return fam.problem(seed), {}


def set_cover_milp(m: int = 200, n: int = 2000, density: float = 0.02, seed: int = 0
                   ) -> tuple[Problem, dict]:
    """0/1 set covering MILP: min cᵀx s.t. A x ≥ 1, x ∈ {0, 1}ⁿ, with A binary
    of the given density (every row covered at least once) and c = U[1, 10];
    the rows are stored as −A x ≤ −1.  Its LP relaxation is fractional and one
    branching step moves the objective by about 0.1–1 %."""
    rng = np.random.default_rng(seed)
    M = rng.random((m, n)) < density
    bare = np.flatnonzero(~M.any(1))
    M[bare, rng.integers(0, n, bare.size)] = True
    A = sp.csr_matrix(M.astype(float))
    p = Problem(c=rng.uniform(1.0, 10.0, n), A_ub=-A, b_ub=-np.ones(m), A_eq=sp.csr_matrix((0, n)),
                b_eq=np.zeros(0), lb=np.zeros(n), ub=np.ones(n), integer_mask=np.ones(n, dtype=bool),
                name=f"setcover_{m}x{n}_s{seed}")
    return p, {}
