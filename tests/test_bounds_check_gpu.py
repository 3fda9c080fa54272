"""Index checks over every kernel family: the library built with -DLQ_BOUNDS_CHECK=1 (each site index
a kernel forms -- neighbours, coordinates -- and each tile plane compared with its bound, a bad one
counted and replaced by 0) runs the HMC path and its companions on lattices that end inside a tile
or a block (L = 2, 3, 5), on the 32^4 and 32^3 index paths and on 48^4, where the per-site kernels
visit their blocks in strips; lq_bounds_check must report the checks on and no bad index.  The
stand-in for a memory checker; the product library is built without the checks."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PKG = os.path.join(REPO, "lattice-qcd-rs_gb300")
CHECKED = os.path.join(PKG, "_build", "checked", "liblqgpu_checked.so")

# run in a child process: the checked library is loaded instead of the product one
SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import lqgpu as G
G.load(sys.argv[2])
assert G.bounds_check(reset=True)[0], "library built without the index checks"
done = []
diverged = []

def traj(s, *args):
    # a projection that diverges (L = 2 lattices, where x + mu and x - mu coincide) or stops at its
    # limit is the reference's own outcome, not an index error
    try:
        s.hmc_trajectory(*args)
    except G.LqError as e:
        if e.code not in (G.LQ_ERR_GAUSS_PROJECTION, G.LQ_ERR_NOT_CONVERGED):
            raise
        diverged.append(e.code)

def state_paths(dim, L, prec):
    with G.State(dim, L, 1000.0, 2.0, prec) as s:
        s.set_links_random(7)
        for k in range(2):
            traj(s, 0.01, 3, 5, k, 0.5)
        s.set_e_field_normal(3, 0, 0.2)
        s.integrate(G.SYNC_SYNC, 0.01, 1)
        s.integrate(G.SYNC_LEAP, 0.01, 1)
        s.integrate(G.LEAP_LEAP, 0.01, 1)
        s.integrate(G.LEAP_SYNC, 0.01, 1)
        s.integrate(G.SYMPLECTIC_EXP, 0.01, 1)
        s.integrate(G.SYMPLECTIC_EXP_REUNITARIZE, 0.01, 1)
        s.simulate_using_leapfrog_n(0.01, 2)
        s.normalize_link_matrices()
        s.hamiltonian_total(); s.average_trace_plaquette(); s.gauss_sum_div(); s.gauss()
        s.wilson_action(); s.wilson_action_backward()
        s.field_strength(); s.magnetic_field()
        if L % 2 == 0:
            s.metropolis_sweep(2, 0.1, 3, 0)
            s.heat_bath_sweep(3, 1)
            s.overrelaxation_sweep(0)
            s.overrelaxation_sweep(1)
        if prec != G.PRECISION_F64 or L <= 5:
            s.leapfrog_adjoint(0.01, 4, 2)
        s.set_link_update(G.LINK_UPDATE_EXP_REUNITARIZE)
        traj(s, 0.01, 2, 5, 9, 0.5)
        c = s.clone(); c.close()
    done.append([dim, L, prec])

for dim in (2, 3, 4):
    for L in (2, 3, 5, 8):
        for prec in (G.PRECISION_F64, G.PRECISION_MIXED, G.PRECISION_F32):
            state_paths(dim, L, prec)
for dim, L in ((3, 32), (4, 32)):
    for prec in (G.PRECISION_MIXED, G.PRECISION_F32):
        with G.State(dim, L, 1000.0, 2.0, prec) as s:
            s.set_links_random(1)
            traj(s, 0.005, 3, 5, 0, 0.5)
        done.append([dim, L, prec])
with G.State(4, 48, 1000.0, 2.0, G.PRECISION_MIXED) as s:
    s.set_links_random(1)
    traj(s, 0.005, 2, 5, 0, 0.5)
done.append([4, 48, 1])
for dim in (2, 3, 4):
    Ls = [2, 3, 5, 8] if dim == 4 else [2, 3, 5, 10]
    for prec in (G.PRECISION_F64, G.PRECISION_MIXED, G.PRECISION_F32):
        with G.Batch(dim, Ls, [1000.0] * 4, [1.5, 2.0, 2.5, 3.0], prec) as b:
            b.set_links_random(2)
            b.set_seed(4, 0)
            b.autotune(0.01, 1)
            b.hmc_run(0.01, 3, 2, 0, graph=True, measure_plaquette=True)
            b.hmc_run(0.01, 3, 1, 0, graph=False)
            b.average_trace_plaquette()
        done.append(["batch", dim, prec])
# the allocation-free plaquette sums (links in the reference layout, device pointers from torch)
import ctypes, torch
lib = G.load()
for dim, L in ((2, 3), (3, 5), (4, 6)):
    links = np.random.default_rng(dim).normal(size=(L ** dim, dim, 18))
    d_links = torch.from_numpy(links).cuda()
    d_out = torch.zeros(3, dtype=torch.float64, device="cuda")
    rc = lib.lq_plaquette_sums_noalloc(dim, L, ctypes.c_void_p(d_links.data_ptr()), ctypes.c_void_p(d_out.data_ptr()),
                                       None)
    assert rc == 0, rc
    torch.cuda.synchronize()
    done.append(["noalloc", dim])
enabled, n, first = G.bounds_check(reset=True)
print(json.dumps({"enabled": enabled, "violations": n, "first_bad": first, "cases": len(done),
                  "diverged": len(diverged)}))
"""


@pytest.fixture(scope="module")
def checked_library():
    sys.path.insert(0, PKG)
    import lqgpu_build

    os.makedirs(os.path.dirname(CHECKED), exist_ok=True)
    lqgpu_build.build(extra=["-DLQ_BOUNDS_CHECK=1"], out=CHECKED)
    return CHECKED


def test_no_index_leaves_its_bounds(checked_library):
    r = subprocess.run([sys.executable, "-c", SCRIPT, PKG, checked_library], capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["enabled"] is True
    assert out["cases"] == 36 + 4 + 1 + 9 + 3
    assert out["violations"] == 0, out
