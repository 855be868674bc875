"""C ABI: the library loads, exports every declared entry point, and its
host-side validation reports malformed input without a GPU."""

import ctypes as C
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp

import sovereign_solver_gb300 as sps
from sovereign_solver_gb300 import _native as N, pdhg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


HEADERS = ("sps_pdhg.h", "sps_gnn.h")


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(sps_[a-z_0-9]+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = N.load()
    names = declared_functions()
    assert len(names) >= 28
    for nm in names:
        assert hasattr(lib, nm), nm


STRUCTS = (("sps_problem_desc", N.ProblemDesc), ("sps_options", N.Options), ("sps_result", N.Result),
           ("sps_batch_stats", N.BatchStats), ("sps_device_lp", N.DeviceLP), ("sps_gnn_graph", N.GnnGraph),
           ("sps_gnn_options", N.GnnOptions))


def test_struct_layout_matches_header(tmp_path):
    """ctypes mirrors agree with a C compiler's view of include/sps_pdhg.h."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    checks = []
    for cname, py in STRUCTS:
        checks.append(f'printf("%s %zu\\n", "{cname}", sizeof({cname}));')
        for fname, _ in py._fields_:
            checks.append(f'printf("%s.%s %zu\\n", "{cname}", "{fname}", offsetof({cname}, {fname}));')
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "sps_pdhg.h"\n#include "sps_gnn.h"\n'
                   'int main(void){' + "".join(checks) + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for cname, py in STRUCTS:
        assert int(got[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)


def test_options_defaults():
    o = pdhg.make_options()
    assert o.mode == 1 and o.precision == 0 and o.max_iters == 100000 and o.tol == 1e-6
    assert o.graph_mode == 2 and o.ruiz_iters == 10
    with pytest.raises(ValueError):
        pdhg.make_options(mode="simplex")
    with pytest.raises(ValueError):
        pdhg.make_options(precision="bf16")


def _lp(**kw):
    p = sps.Problem(c=np.array([1.0, 2.0]), A_ub=sp.csr_matrix(np.array([[-1.0, -1.0]])),
                    b_ub=np.array([-2.0]), A_eq=sp.csr_matrix((0, 2)), b_eq=np.zeros(0),
                    lb=np.zeros(2), ub=np.full(2, np.inf), integer_mask=np.zeros(2, bool))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("bad,msg", [
    (dict(c=np.array([np.nan, 1.0])), "objective"),
    (dict(b_ub=np.array([np.inf])), "right-hand side"),
    (dict(lb=np.array([1.0, 0.0]), ub=np.array([0.0, 1.0])), "bounds"),
    (dict(lb=np.array([np.inf, 0.0])), "bounds"),
])
def test_invalid_input_raises_valueerror_before_device_use(bad, msg):
    with pytest.raises(ValueError, match=msg):
        pdhg.solve_lp_pdhg(_lp(**bad))


def test_bad_column_index_is_rejected():
    p = _lp()
    A = p.A_ub.copy()
    A.indices = A.indices.copy()
    A.indices[0] = 7                       # out of range; caught on the device or with no device
    p.A_ub = A
    with pytest.raises((ValueError, RuntimeError)):
        pdhg.solve_lp_pdhg(p)


def test_unknown_device_and_method():
    with pytest.raises(ValueError):
        sps.solve_lp_pdhg_gpu(_lp(), device="mps")
    with pytest.raises(ValueError):
        sps.Solver().set_problem(_lp()).solve(method="simplex")
    with pytest.raises(RuntimeError):
        sps.Solver().solve(method="pdhg")


def test_kkt_form_rejected_where_it_does_not_apply():
    """The PDLP error form is an option of the adaptive single-LP engine: the
    reference mode and the batched solver reject it before any device work."""
    p = _lp()
    with pytest.raises(ValueError, match="kkt_form"):
        pdhg.solve_lp_pdhg(p, mode="reference", kkt_form="pdlp")
    with pytest.raises(ValueError, match="kkt_form"):
        pdhg.solve_lp_pdhg(p, kkt_form="strict")
    with pytest.raises(ValueError, match="Lagrangian"):
        sps.PDHGBatch([p, p], kkt_form="pdlp")


def test_get_available_device_values():
    assert sps.get_available_device() in ("cuda", "cpu")


@pytest.mark.skipif(pdhg.get_available_device() == "cuda", reason="checks the no-GPU error path")
def test_no_gpu_fails_loudly():
    with pytest.raises(RuntimeError, match="CUDA"):
        pdhg.solve_lp_pdhg(_lp())


def test_integration_stub_matches_the_abi():
    """The ctypes stub a maintainer would paste into the reference tree
    (``tests/integration_stub.py`` holds its struct declarations) declares the
    same struct layouts as the package's own binding, which the test above
    checks against the header."""
    import integration_stub as stub_mod
    for stub, ours in ((stub_mod.Desc, N.ProblemDesc), (stub_mod.Opts, N.Options), (stub_mod.Res, N.Result)):
        assert C.sizeof(stub) == C.sizeof(ours), stub.__name__
        assert [f for f, _ in stub._fields_] == [f for f, _ in ours._fields_], stub.__name__
        for f, _ in stub._fields_:
            assert getattr(stub, f).offset == getattr(ours, f).offset, (stub.__name__, f)


def test_gather_floor_rejects_bad_arguments():
    """The gather-floor benchmark checks its arguments before any device work."""
    lib = N.load()
    out = np.zeros(2)
    for args in ((0, 10, 1), (100, 0, 1), (100, 10, 0)):
        assert lib.sps_time_gather_floor(args[0], args[1], args[2], 0, N.f64p(out)) == -1
    assert lib.sps_time_gather_floor(100, 10, 1, 0, None) == -1


def test_create_validation_names_the_first_bad_variable():
    """sps_create's validation scans (on the set-up's host worker pool for large
    inputs) report the first invalid variable whichever thread's chunk finds it;
    the call returns before any device work, so it runs without a GPU."""
    import ctypes as C
    from sovereign_solver_gb300 import _native as N
    n = 300_000
    lb, ub = np.zeros(n), np.full(n, np.inf)
    lb[[250_000, 200_123, 299_999]] = [5.0, 3.0, np.inf]      # lb > ub, lb > ub, lb = +inf
    ub[[250_000, 200_123]] = 1.0
    p = sps.Problem(c=np.ones(n), A_ub=sp.csr_matrix((np.ones(n), (np.zeros(n, int), np.arange(n))), shape=(1, n)),
                    b_ub=np.array([1.0]), A_eq=sp.csr_matrix((0, n)), b_eq=np.zeros(0), lb=lb, ub=ub,
                    integer_mask=np.zeros(n, bool))
    lib = N.load()
    d = pdhg._Desc(p)
    h = C.c_void_p()
    for _ in range(3):                                        # the pool is reused between calls
        rc = lib.sps_create(C.byref(d.desc), C.byref(pdhg.make_options()), C.byref(h))
        assert rc == -1 and not h.value
        assert lib.sps_last_error(None).decode() == "invalid bounds at variable 200123"
