"""The set-up's host worker pool (csrc/host_pool.cuh), checked on the CPU through
a host-only helper (tests/pool_check.cpp): every chunk of every loop runs exactly
once, with concurrent callers, with a loop started from inside a pool task, and
in a child process forked after the pool started."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_host_pool(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "pool_check")
    cmd = [cxx, "-std=c++17", "-O1", "-pthread", "-x", "c++",
           f"-I{os.path.join(ROOT, 'sovereign-solver_gb300', 'csrc')}", os.path.join(HERE, "pool_check.cpp"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    lines = r.stdout.split("\n")
    for check in ("loops", "callers", "nested", "fork"):
        assert f"{check} ok" in lines, r.stdout + r.stderr
    assert r.returncode == 0, r.stdout + r.stderr
