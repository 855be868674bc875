"""The warm-start network's CPU oracle: its analytic backward pass agrees with
central finite differences (exact weights, FP64), and its BF16 rounding is
round-to-nearest-even."""

import numpy as np
import scipy.sparse as sp

from oracle import gnn_ref


def _case(seed=0, n=11, m=5, H=4, L=2, Fv=2, Fc=3, B=2):
    rng = np.random.default_rng(seed)
    A = sp.random(m, n, density=0.4, random_state=seed, format="csr")
    A.data = rng.standard_normal(A.nnz)
    lay = gnn_ref.Layout(H, L, Fv, Fc)
    p = rng.standard_normal(lay.size) * 0.5
    fvs = [rng.standard_normal((n, Fv)) for _ in range(B)]
    fcs = [rng.standard_normal((m, Fc)) for _ in range(B)]
    xts = [rng.standard_normal(n) for _ in range(B)]
    yts = [rng.standard_normal(m) for _ in range(B)]
    lts = list(rng.standard_normal(B))
    return lay, p, (A.indptr, A.indices, A.data), fvs, fcs, xts, yts, lts


def test_backward_matches_finite_differences():
    lay, p, g, fvs, fcs, xts, yts, lts = _case()
    f0, grad = gnn_ref.loss_grad(p, lay, *g, fvs, fcs, xts, yts, lts, bf16=False)
    rng = np.random.default_rng(1)
    idx = rng.choice(lay.size, size=60, replace=False)
    eps = 1e-6
    for k in idx:
        e = np.zeros(lay.size)
        e[k] = eps
        fp, _ = gnn_ref.loss_grad(p + e, lay, *g, fvs, fcs, xts, yts, lts, bf16=False)
        fm, _ = gnn_ref.loss_grad(p - e, lay, *g, fvs, fcs, xts, yts, lts, bf16=False)
        fd = (fp - fm) / (2 * eps)
        assert abs(fd - grad[k]) <= 1e-6 * (1 + abs(fd)), (k, fd, grad[k])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159265], np.float32)
    r = gnn_ref.bf16_round(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                       # halfway 1 + 2^-8: ties to even (1.0)
    assert r[2] == 1.0 + 2 ** -7             # above halfway rounds up
    assert r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-12
