"""The launch order of the per-site stencil kernels' blocks (lattice-qcd-rs_gb300/csrc/block_order.hpp)
is a permutation of the blocks for every lattice shape, strip-mined or not: compiled and run on the
host (the header is plain C++ outside nvcc)."""
import os
import subprocess

from conftest import PKG, REPO

SRC = os.path.join(REPO, "tests", "cpp", "test_block_order.cpp")


def test_block_order_is_a_permutation(tmp_path):
    exe = os.path.join(str(tmp_path), "test_block_order")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(PKG, "csrc"), SRC, "-o",
           exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "PASSED" in r.stdout, r.stdout + r.stderr
