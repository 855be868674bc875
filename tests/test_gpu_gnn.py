"""Warm-start network on the GPU: forward outputs and gradients of the
hand-written kernels against the FP64 CPU oracle (same BF16 weight rounding),
and a short training run that lowers the loss and is bitwise reproducible."""

import numpy as np
import pytest
import scipy.sparse as sp

import sovereign_solver_gb300 as sps
from sovereign_solver_gb300.gnn import WarmStartGNN
from oracle import gnn_ref

pytestmark = pytest.mark.gpu


def _template(n=300, m=40, m_ub=15, seed=0):
    rng = np.random.default_rng(seed)
    A = sp.random(m, n, density=0.06, random_state=seed, format="csr")
    A.data = rng.standard_normal(A.nnz)
    return sps.Problem(c=rng.random(n), A_ub=A[:m_ub], b_ub=rng.random(m_ub) + 1, A_eq=A[m_ub:],
                       b_eq=rng.random(m - m_ub), lb=np.zeros(n), ub=np.full(n, np.inf),
                       integer_mask=np.zeros(n, bool), name="gnn_template")


def _data(net, B, seed=1):
    rng = np.random.default_rng(seed)
    fvs = [rng.standard_normal((net.n, 4)).astype(np.float32) for _ in range(B)]
    fcs = [rng.standard_normal((net.m, 4)).astype(np.float32) for _ in range(B)]
    xts = [rng.random(net.n).astype(np.float32) for _ in range(B)]
    yts = [rng.standard_normal(net.m).astype(np.float32) for _ in range(B)]
    lts = rng.standard_normal(B).astype(np.float32)
    return fvs, fcs, xts, yts, lts


@pytest.mark.parametrize("hidden", [64, 32])
def test_gradients_match_oracle(hidden):
    p = _template()
    with WarmStartGNN(p, hidden=hidden, layers=3, seed=3, max_batch=4, lp_features=False) as net:
        fvs, fcs, xts, yts, lts = _data(net, 3)
        loss, g = net.loss_grad(fvs, fcs, xts, yts, lts)
        params = net.params()
        lay = gnn_ref.Layout(hidden, 3, 4, 4)
        assert lay.size == net.num_params
        ref_loss, ref_g = gnn_ref.loss_grad(params, lay, net._ptr, net._idx, net._val, fvs, fcs, xts, yts,
                                            list(lts), 1.0, 1.0, 0.1, bf16=True)
    assert abs(loss - ref_loss) <= 1e-5 * (1 + abs(ref_loss)), (loss, ref_loss)
    assert np.linalg.norm(g - ref_g) <= 1e-4 * np.linalg.norm(ref_g)
    for name, o, shape, _ in lay.items:          # every parameter block
        k = int(np.prod(shape))
        ref = ref_g[o:o + k]
        assert np.linalg.norm(g[o:o + k] - ref) <= 2e-3 * np.linalg.norm(ref) + 1e-7, name


def test_forward_matches_oracle():
    p = _template(seed=4)
    with WarmStartGNN(p, seed=5, max_batch=2, lp_features=False) as net:
        fvs, fcs, *_ = _data(net, 2, seed=6)
        X, Y, Lw = net.predict_features(fvs, fcs)
        lay = gnn_ref.Layout(64, 3, 4, 4)
        params = net.params()
        for s in range(2):
            x, y, lw = gnn_ref.predict(params, lay, net._ptr, net._idx, net._val, fvs[s], fcs[s])
            np.testing.assert_allclose(X[s], x, rtol=1e-4, atol=1e-5 * np.abs(x).max())
            np.testing.assert_allclose(Y[s], y, rtol=1e-4, atol=1e-5 * np.abs(y).max())
            assert abs(Lw[s] - lw) <= 1e-4 * (1 + abs(lw))


def test_training_lowers_loss_and_is_reproducible():
    p = _template(seed=7)
    runs = []
    for _ in range(2):
        with WarmStartGNN(p, seed=11, lr=3e-3, max_batch=4, lp_features=False) as net:
            fvs, fcs, xts, yts, lts = _data(net, 4, seed=8)
            losses = [net.train_step(fvs, fcs, xts, yts, lts) for _ in range(150)]
            runs.append((losses, net.params()))
    (l1, p1), (l2, p2) = runs
    assert l1[-1] < 0.5 * l1[0], (l1[0], l1[-1])
    assert l1 == l2
    np.testing.assert_array_equal(p1, p2)


def test_batch_limit_and_bad_params():
    p = _template()
    with WarmStartGNN(p, max_batch=2, lp_features=False) as net:
        fvs, fcs, xts, yts, lts = _data(net, 3)
        with pytest.raises(RuntimeError):
            net.train_step(fvs, fcs, xts, yts, lts)
        bad = net.params()
        bad[0] = np.nan
        with pytest.raises(RuntimeError):
            net.set_params(bad)


def test_device_lp_features_match_host_features():
    """lp_features: the device expansion of (c, b) gives the predictions of the NumPy features."""
    p = _template(seed=9)
    rng = np.random.default_rng(10)
    cs = [rng.random(p.n_vars) + 0.1 for _ in range(3)]
    bs = [rng.random(p.n_ineq + p.n_eq) + 0.5 for _ in range(3)]
    with WarmStartGNN(p, seed=12, max_batch=4, lp_features=True) as dev, \
            WarmStartGNN(p, seed=12, max_batch=4, lp_features=False, scales=dev.scales) as host:
        np.testing.assert_array_equal(dev.params(), host.params())
        fd = [dev.features_from(c, b) for c, b in zip(cs, bs)]
        assert fd[0][0].shape == (p.n_vars, 1) and fd[0][1].shape == (p.n_ineq + p.n_eq, 1)
        fh = [host.host_features(c, b) for c, b in zip(cs, bs)]
        Xd, Yd, Ld = dev.predict_features([f[0] for f in fd], [f[1] for f in fd])
        Xh, Yh, Lh = host.predict_features([f[0] for f in fh], [f[1] for f in fh])
    np.testing.assert_allclose(Xd, Xh, rtol=1e-4, atol=1e-5 * np.abs(Xh).max())
    np.testing.assert_allclose(Yd, Yh, rtol=1e-4, atol=1e-5 * np.abs(Yh).max())
    np.testing.assert_allclose(Ld, Lh, rtol=1e-4, atol=1e-5)
