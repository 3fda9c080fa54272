"""The C++ host interface that mirrors the reference's types (LatticeStateDefault,
LatticeStateEFSyncDefault, SymplecticIntegrator, HybridMonteCarloDiagnostic): it compiles
against the C ABI header on any machine, and its test program runs on the GPU."""
import os
import subprocess

import pytest

from conftest import PKG, REPO

SRC = os.path.join(REPO, "tests", "cpp", "test_host_mirror.cpp")


def compile_program(lqgpu_mod, out_dir):
    exe = os.path.join(out_dir, "test_host_mirror")
    lib_dir = os.path.dirname(lqgpu_mod.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"),
           "-I", os.path.join(PKG, "host"), SRC, "-o", exe, "-L", lib_dir, "-llqgpu", "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_host_mirror_compiles(lqgpu_mod, tmp_path):
    assert os.path.exists(compile_program(lqgpu_mod, str(tmp_path)))


@pytest.mark.gpu
def test_host_mirror_program(lqgpu_mod, tmp_path):
    exe = compile_program(lqgpu_mod, str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout
