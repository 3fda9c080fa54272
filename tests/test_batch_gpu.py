"""Batched ensembles (lq_batch_*): many lattices of uneven side length and beta advanced by
one launch per kernel of a trajectory, replayed as a CUDA graph with the Gauss projection's
sweep loop as a device-side while node.

Each ensemble of a batch must evolve exactly as a state of the same precision run alone
through lq_hmc_trajectory with the same seed (batch seed + ensemble index), counter and
accept uniform: the per-link arithmetic is shared, so the links after K trajectories are
bitwise equal for the FP32-arithmetic forms (both use the fused projection sweep) and equal
to 1e-12 for FP64 (the state projects with two kernels per step, the batch with the fused
sweep).  Delta H is compared to 1e-9 relative to the link Hamiltonian: the state forms it
as a difference of two Hamiltonians (FP64) or of Hamiltonian updates, the batch from the
difference kernels directly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIM = 4
LS = [3, 4, 5, 4, 3]
BETAS = [1.5, 2.0, 3.0, 2.5, 6.0]
SIZES = [1000.0, 1000.0, 1000.0, 20.0, 1000.0]
SEED, LINK_SEED = 77, 5
DT, NSTEPS, NTRAJ, MAXG = 0.01, 6, 4, 10001


def make_batch(G, precision, Ls=LS, betas=BETAS, sizes=SIZES):
    b = G.Batch(DIM, Ls, sizes, betas, precision)
    b.set_links_random(LINK_SEED)
    b.set_seed(SEED, 0)
    return b


@pytest.mark.parametrize("precision", [1, 2, 0])
def test_batch_matches_single_lattice_runs(lqgpu_mod, precision):
    G = lqgpu_mod
    with make_batch(G, precision) as b:
        b.hmc_run(DT, NSTEPS, NTRAJ, MAXG, graph=True)
        res = b.hmc_results()
        links_b = [b.link_matrix(e) for e in range(b.n)]
    assert (res["status"] == 0).all()
    for e, (L, beta, size) in enumerate(zip(LS, BETAS, SIZES)):
        with G.State(DIM, L, size, beta, precision) as s:
            s.set_links_random(LINK_SEED + e)
            hu = s.hamiltonian_links()
            for k in range(NTRAJ):
                r = s.hmc_trajectory(DT, NSTEPS, SEED + e, k, float(res["uniform"][k, e]), MAXG)
                assert r["gauss_steps"] == res["gauss_steps"][k, e]
                assert r["accepted"] == res["accepted"][k, e]
                assert abs(r["delta_h"] - res["delta_h"][k, e]) <= 1e-9 * max(1.0, hu)
            if precision == 0:
                assert np.abs(s.link_matrix() - links_b[e]).max() <= 1e-12
            else:
                assert np.array_equal(s.link_matrix(), links_b[e])


def test_graph_replay_equals_eager_launches(lqgpu_mod):
    G = lqgpu_mod
    out = []
    for graph in (True, False):
        with make_batch(G, G.PRECISION_MIXED) as b:
            b.hmc_run(DT, NSTEPS, NTRAJ, MAXG, graph=graph, measure_plaquette=True)
            out.append((b.hmc_results(), [b.link_matrix(e) for e in range(b.n)], b.graph_launches()))
    (ra, la, na), (rb, lb, nb) = out
    assert na == NTRAJ and nb == 0
    for key in ("delta_h", "accepted", "gauss_steps", "uniform", "plaquette"):
        assert np.array_equal(ra[key], rb[key]), key
    for x, y in zip(la, lb):
        assert np.array_equal(x, y)


def test_results_do_not_depend_on_tuned_launch_shapes(lqgpu_mod):
    G = lqgpu_mod
    runs = []
    for tune in (False, True):
        with make_batch(G, G.PRECISION_MIXED) as b:
            if tune:
                t = b.autotune(DT, 2)
                assert all(v["ms"] > 0.0 for v in t.values())
            b.hmc_run(DT, NSTEPS, 2, MAXG)
            runs.append((b.hmc_results(), [b.link_matrix(e) for e in range(b.n)]))
    for key in ("delta_h", "accepted", "gauss_steps", "uniform", "prob"):
        assert np.array_equal(runs[0][0][key], runs[1][0][key]), key
    for x, y in zip(runs[0][1], runs[1][1]):
        assert np.array_equal(x, y)


def test_persistent_grids_give_the_same_links(lqgpu_mod):
    """Tuning picks grids of a few waves for the larger batch; links equal the untuned run."""
    G = lqgpu_mod
    Ls, betas, sizes = [6, 8, 7, 5, 8, 6], [2.0, 2.5, 3.0, 1.5, 4.0, 2.2], [1000.0] * 6
    runs = []
    for tune in (False, True):
        with make_batch(G, G.PRECISION_F32, Ls, betas, sizes) as b:
            if tune:
                b.autotune(DT, 1)
            b.hmc_run(DT, 3, 2, MAXG)
            runs.append([b.link_matrix(e) for e in range(b.n)])
    for x, y in zip(*runs):
        assert np.array_equal(x, y)


def test_step_limit_keeps_links_and_reports_status(lqgpu_mod):
    G = lqgpu_mod
    with make_batch(G, G.PRECISION_MIXED) as b:
        before = [b.link_matrix(e) for e in range(b.n)]
        b.hmc_run(DT, NSTEPS, 2, max_gauss_steps=2)
        r = b.hmc_results()
        after = [b.link_matrix(e) for e in range(b.n)]
    # a random draw is not projected after one step: every ensemble stops at the limit
    assert (r["status"] == G.LQ_ERR_NOT_CONVERGED).all()
    assert not r["accepted"].any()
    for x, y in zip(before, after):
        assert np.array_equal(x, y)


def test_recorded_plaquette_and_batch_observables(lqgpu_mod):
    G = lqgpu_mod
    with make_batch(G, G.PRECISION_MIXED) as b:
        b.hmc_run(DT, NSTEPS, 3, MAXG, measure_plaquette=True)
        r = b.hmc_results()
        plaq = b.average_trace_plaquette()
        links = [b.link_matrix(e) for e in range(b.n)]
    assert np.array_equal(r["plaquette"][-1], plaq.real)
    for e, (L, beta, size) in enumerate(zip(LS, BETAS, SIZES)):
        with G.State(DIM, L, size, beta, G.PRECISION_F64) as s:
            s.set_link_matrix(links[e])
            assert abs(s.average_trace_plaquette() - plaq[e]) <= 1e-6


def test_uneven_batch_dims_2_and_3(lqgpu_mod):
    G = lqgpu_mod
    for dim, Ls in ((2, [5, 9, 4]), (3, [3, 6, 4])):
        with G.Batch(dim, Ls, [1000.0] * 3, [2.0, 3.0, 4.0], G.PRECISION_MIXED) as b:
            b.set_links_random(3)
            b.set_seed(11, 0)
            b.hmc_run(0.02, 4, 2, MAXG)
            res = b.hmc_results()
            links = [b.link_matrix(e) for e in range(3)]
        for e, L in enumerate(Ls):
            with G.State(dim, L, 1000.0, [2.0, 3.0, 4.0][e], G.PRECISION_MIXED) as s:
                s.set_links_random(3 + e)
                for k in range(2):
                    r = s.hmc_trajectory(0.02, 4, 11 + e, k, float(res["uniform"][k, e]), MAXG)
                    assert r["accepted"] == res["accepted"][k, e]
                assert np.array_equal(s.link_matrix(), links[e])


@pytest.mark.parametrize("precision", [1, 0])
def test_tiny_and_ragged_ensembles(lqgpu_mod, precision):
    """L = 2 (x + mu and x - mu coincide) and volumes that end inside a tile (3^4 = 81, 5^4 = 625
    sites) next to each other in one batch; a batch of one ensemble."""
    G = lqgpu_mod
    for Ls, betas in (([2, 3, 2, 5], [2.0, 3.0, 4.0, 2.5]), ([3], [2.0])):
        n = len(Ls)
        with G.Batch(DIM, Ls, [1000.0] * n, betas, precision) as b:
            b.set_links_random(21)
            b.set_seed(5, 0)
            b.hmc_run(DT, 4, 2, MAXG)
            res = b.hmc_results()
            links = [b.link_matrix(e) for e in range(n)]
        assert (res["status"] == 0).all()
        for e, (L, beta) in enumerate(zip(Ls, betas)):
            with G.State(DIM, L, 1000.0, beta, precision) as s:
                s.set_links_random(21 + e)
                for k in range(2):
                    r = s.hmc_trajectory(DT, 4, 5 + e, k, float(res["uniform"][k, e]), MAXG)
                    assert r["accepted"] == res["accepted"][k, e]
                    assert r["gauss_steps"] == res["gauss_steps"][k, e]
                if precision == 0:
                    assert np.abs(s.link_matrix() - links[e]).max() <= 1e-12
                else:
                    assert np.array_equal(s.link_matrix(), links[e])


def test_eager_kernel_profile_counts_every_launch(lqgpu_mod):
    """the kernel-time profile of eager trajectories sees every launch, none inside a graph"""
    G = lqgpu_mod
    with make_batch(G, G.PRECISION_MIXED) as b:
        b.profile_enable(True)
        b.hmc_run(DT, NSTEPS, 1, MAXG, graph=True)
        assert b.profile_read(reset=True) == (0, 0.0)
        b.hmc_run(DT, NSTEPS, 2, MAXG, graph=False)
        n, ms = b.profile_read(reset=True)
        steps = b.hmc_results()["gauss_steps"].max(axis=1)
        # per trajectory: draw, Gauss law, the sweeps and their checks (one per 1 or 4 sweeps),
        # the compensated zeroing, NSTEPS + 1 MD launches, two difference kernels, the accept
        expected = sum(2 + int(k) + 1 + (int(k) - 1) // 4 + 1 + NSTEPS + 1 + 3 for k in steps)
        assert n == expected, (n, expected)
        assert ms > 0.0
        b.profile_enable(False)


@pytest.mark.parametrize("dim,L", [(2, 32), (3, 32), (4, 32), (4, 48), (2, 16), (3, 8), (4, 8)])
def test_lone_state_at_L32_equals_batched_ensemble(lqgpu_mod, dim, L):
    """the headline's side length: a lone mixed state and the same lattice as a one-ensemble batch
    (the batch's persistent kernels over a chunk table) give the same accept decisions, projection
    steps and links, bitwise.  At 48^4 the lone state's MD and sweep kernels visit their blocks in
    strips (block_order.hpp) while the batch's run in site order; where L divides 32 (32, 16, 8: one
    or several lattice rows per warp) the lone state's sweep takes the direction-0 neighbour's step
    by shuffle while the batch's recomputes it."""
    G = lqgpu_mod
    with G.Batch(dim, [L], [1000.0], [2.0], G.PRECISION_MIXED) as b:
        b.set_links_random(LINK_SEED)
        b.set_seed(SEED, 0)
        b.hmc_run(DT, 3, 2, MAXG)
        rb = b.hmc_results()
        links_b = b.link_matrix(0)
    with G.State(dim, L, 1000.0, 2.0, G.PRECISION_MIXED) as s:
        s.set_links_random(LINK_SEED)
        for k in range(2):
            r = s.hmc_trajectory(DT, 3, SEED, k, float(rb["uniform"][k, 0]))
            assert r["accepted"] == bool(rb["accepted"][k, 0])
            assert r["gauss_steps"] == rb["gauss_steps"][k, 0]
        assert np.array_equal(s.link_matrix(), links_b)
