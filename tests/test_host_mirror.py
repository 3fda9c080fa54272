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


DRIVER = os.path.join(PKG, "host", "hmc_driver_timing.cpp")


def compile_driver_timing(lqgpu_mod, out_dir):
    exe = os.path.join(out_dir, "hmc_driver_timing")
    lib_dir = os.path.dirname(lqgpu_mod.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"),
           "-I", os.path.join(PKG, "host"), DRIVER, "-o", exe, "-L", lib_dir, "-llqgpu", "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_driver_timing_program_compiles(lqgpu_mod, tmp_path):
    """the bench's C++ HybridMonteCarloDiagnostic timing program builds against the header"""
    exe = compile_driver_timing(lqgpu_mod, str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
def test_driver_timing_program_runs(lqgpu_mod, tmp_path):
    import json

    exe = compile_driver_timing(lqgpu_mod, str(tmp_path))
    r = subprocess.run([exe, "6", "3", "1", "1", "10", "0.01", "2.0"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["value"] > 0 and out["trajectories"] == 3 and 0 <= out["accepted"] <= 3
