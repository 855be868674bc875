"""sps_kkt_noalloc: the KKT check that allocates no device memory.

Some callers cannot call cudaMalloc when they want a point checked: code that
runs inside another framework's memory pool or a fixed device-memory budget,
or a latency-critical loop where an allocation would synchronise the device.
For them the library offers one entry point whose scratch is a fixed array
inside the library; they pass the LP, the point and an output buffer, all in
device memory they already own.

The GPU test checks it, through the C ABI, twice in a row, against what the
existing entry point sps_solve reports for the same point (same tolerance form
as the other parity tests: 0.5 * tol absolute + 1e-3 relative, since sps_solve
evaluates with the FP32-rounded scaled matrix) and against the CPU oracle's FP64
evaluation (1e-9 relative plus 1e-12 absolute: both are FP64 sums of the same
products, in different orders).  Its K^T y is summed with integer digits, so
the two calls must agree bit for bit, on LPs whose columns hold 2 (transport),
about 10 (planted 200x500) and about 40 (planted 2000x4000) nonzeros; free
device memory must not change across calls.  This file is collected last.
"""

import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

import sovereign_solver_gb300 as sps
import sovereign_solver_gb300.workloads as wl
from sovereign_solver_gb300 import _native as N
from fixtures import load_problems
from oracle import kkt

TOL = 1e-5


def _case(name):
    if name == "planted":
        return wl.planted_lp(seed=11)[0]
    if name == "planted_dense":
        return wl.planted_lp(m=2000, n=4000, density=0.02, seed=3)[0]
    if name == "transport":
        return wl.transportation_lp(30, 60, seed=2)[0]
    return load_problems()["mixed_bounds"]


def _device_lp(torch, p):
    K = sp.vstack([sp.csr_matrix(p.A_ub, dtype=float), sp.csr_matrix(p.A_eq, dtype=float)], format="csr")
    rhs = np.concatenate([np.asarray(p.b_ub, float), np.asarray(p.b_eq, float)])
    dev = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    keep = [dev(K.indptr.astype(np.int32), torch.int32), dev(K.indices.astype(np.int32), torch.int32),
            dev(K.data, torch.float64), dev(p.c, torch.float64), dev(rhs, torch.float64),
            dev(p.lb, torch.float64), dev(p.ub, torch.float64)]
    lp = N.DeviceLP(p.n_vars, p.n_ineq, p.n_eq, *[t.data_ptr() for t in keep])
    return lp, keep


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["planted", "planted_dense", "transport", "mixed_bounds"])
def test_noalloc_kkt_matches_sps_solve(name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    p = _case(name)
    with sps.PDHGEngine(p, tol=TOL, max_iters=200000) as eng:
        r = eng.solve_raw()
        x, y = eng.solution()
    assert r.status == 0
    lib = N.load()
    lp, keep = _device_lp(torch, p)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    yd = torch.tensor(y, dtype=torch.float64, device="cuda")
    out = torch.empty(6, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        out.fill_(float("nan"))
        rc = lib.sps_kkt_noalloc(C.byref(lp), xd.data_ptr(), yd.data_ptr(), out.data_ptr(), stream)
        assert rc == 0, lib.sps_last_error(None)
        torch.cuda.synchronize()
        return out.cpu().numpy().copy()

    call()      # the library's device module (and its static scratch) may load lazily on first use
    free0 = torch.cuda.mem_get_info()[0]
    calls = [call(), call()]
    assert torch.cuda.mem_get_info()[0] == free0, "free device memory changed across calls"
    engine = np.array([r.rel_kkt, r.rel_primal, r.rel_dual, r.rel_gap])
    box = kkt.box_rel_kkt(p, x, y)
    ref = np.array([box["err"], box["rp"], box["rd"], box["gap"], box["pobj"], box["dobj"]])
    for got in calls:
        assert np.all(np.isfinite(got))
        assert np.all(np.abs(got[:4] - engine) <= 0.5 * TOL + 1e-3 * np.abs(engine)), (got[:4], engine)
        np.testing.assert_allclose(got[:4], ref[:4], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(got[4:], ref[4:], rtol=1e-9, atol=1e-12)
    assert np.array_equal(calls[0], calls[1]), calls


def test_noalloc_rejects_too_many_columns():
    """More columns than the fixed scratch holds: a clear error, no device work."""
    lib = N.load()
    lp = N.DeviceLP(300000, 0, 1, 8, 8, 8, 8, 8, 8, 8)
    rc = lib.sps_kkt_noalloc(C.byref(lp), 8, 8, 8, None)
    assert rc == -1
    assert b"262144" in lib.sps_last_error(None)


@pytest.mark.parametrize("missing", ["indptr", "indices", "values", "rhs", "c", "lb", "ub"])
def test_noalloc_rejects_null_arrays(missing):
    """A null device array where the LP needs one: a clear error before any device work
    (rows need indptr, indices, values and rhs even when they hold no nonzeros)."""
    lib = N.load()
    lp = N.DeviceLP(4, 1, 1, 8, 8, 8, 8, 8, 8, 8)
    setattr(lp, missing, None)
    rc = lib.sps_kkt_noalloc(C.byref(lp), 8, 8, 8, None)
    assert rc == -1
    assert b"null device array" in lib.sps_last_error(None)
