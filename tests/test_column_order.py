"""The engine's host ordering of CSC columns too long for the device insertion
sort (more than 64 entries), checked on the CPU through a host-only helper
(tests/colsort_dump.cu): every long column of the range comes back ordered by
row index with its values alongside, every shorter column untouched, over
ranges with few and with many (threaded) long columns."""

import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SORT_MAX = 64


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("colsort") / "colsort_dump")
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
           f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(ROOT, 'sovereign-solver_gb300', 'csrc')}",
           os.path.join(HERE, "colsort_dump.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.mark.parametrize("ncols,seed", [(300, 0), (12000, 1)])
def test_long_columns_ordered(tool, tmp_path, ncols, seed):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 130, ncols)
    lens[rng.random(ncols) < 0.02] = rng.integers(1000, 3000)
    cptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = np.concatenate([rng.permutation(5000)[:k] for k in lens]).astype(np.int32)
    val = rng.standard_normal(idx.size)
    j0, j1 = 3, ncols - 2
    lo, hi = cptr[j0], cptr[j1]
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        f.write(struct.pack("<iii", ncols, j0, j1))
        f.write(cptr.tobytes())
        f.write(idx[lo:hi].tobytes())
        f.write(val[lo:hi].tobytes())
    subprocess.run([tool, fin, fout], check=True)
    raw = open(fout, "rb").read()
    got_i = np.frombuffer(raw[:4 * (hi - lo)], np.int32)
    got_v = np.frombuffer(raw[4 * (hi - lo):], np.float64)
    for j in range(j0, j1):
        s, t = cptr[j] - lo, cptr[j + 1] - lo
        want_i, want_v = idx[cptr[j]:cptr[j + 1]], val[cptr[j]:cptr[j + 1]]
        if t - s > SORT_MAX:
            o = np.argsort(want_i, kind="stable")
            want_i, want_v = want_i[o], want_v[o]
        np.testing.assert_array_equal(got_i[s:t], want_i)
        np.testing.assert_array_equal(got_v[s:t], want_v)
