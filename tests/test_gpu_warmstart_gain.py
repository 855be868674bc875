"""What the trained warm-start network gains over the method without it.

The committed weights (trained by ``sovereign-solver_gb300/warmstart.py`` on
seeds 0..19 999 of the 200 x 400 transportation family) predict warm starts for
held-out seeds; the warm-started batched solves need far fewer iterations than
the same solves from zero, and every answer passes the FP64 KKT check."""

import os

import numpy as np
import pytest

import sovereign_solver_gb300 as sps
from sovereign_solver_gb300.gnn import WarmStartGNN
from sovereign_solver_gb300.warmstart import transport_instances
from sovereign_solver_gb300.workloads import TransportFamily
from oracle import kkt

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WEIGHTS = os.path.join(ROOT, "sovereign-solver_gb300", "data", "warmstart_transport_200x400.npz")
TOL = 1e-4


def test_learned_warm_start_gain_on_held_out_seeds():
    fam = TransportFamily()
    template = fam.problem(0)
    probs = transport_instances(fam, template, range(20_000_000, 20_000_048))
    with WarmStartGNN.load(WEIGHTS, template, max_batch=16) as net, sps.PDHGBatch(probs, tol=TOL) as b:
        cold = b.solve()
        b.set_warm_starts(net.predict(probs))
        warm = b.solve()
    ci = np.array([r.iterations for r in cold], float)
    wi = np.array([r.iterations for r in warm], float)
    used = sum(r.stats["warm_start_used"] for r in warm)
    print(f"cold mean {ci.mean():.0f} it, warm mean {wi.mean():.0f} it, warm starts used {used}/{len(probs)}")
    assert used >= 0.9 * len(probs)
    assert wi.mean() <= 0.75 * ci.mean()
    for p, r in zip(probs, warm):
        assert r.status == "optimal"
        assert kkt.box_rel_kkt(p, r.x, r.y)["err"] < 1.5 * TOL


def test_device_predicted_warm_starts():
    """The same network predicting on the device straight into the batch's
    warm-start buffers (sps_batch_set_warm_starts_gnn) gives the same gain."""
    fam = TransportFamily()
    template = fam.problem(0)
    probs = transport_instances(fam, template, range(20_000_100, 20_000_140))
    with WarmStartGNN.load(WEIGHTS, template, max_batch=16) as net, sps.PDHGBatch(probs, tol=TOL) as b:
        cold = b.solve()
        b.set_warm_starts_gnn(net)
        warm = b.solve()
        b.set_warm_starts(net.predict(probs))      # host path, for comparison
        host = b.solve()
    ci = np.array([r.iterations for r in cold], float)
    wi = np.array([r.iterations for r in warm], float)
    hi = np.array([r.iterations for r in host], float)
    assert sum(r.stats["warm_start_used"] for r in warm) >= 0.9 * len(probs)
    assert wi.mean() <= 0.75 * ci.mean()
    assert abs(wi.mean() - hi.mean()) <= 0.1 * hi.mean()
    for p, r in zip(probs, warm):
        assert r.status == "optimal"
        assert kkt.box_rel_kkt(p, r.x, r.y)["err"] < 1.5 * TOL
