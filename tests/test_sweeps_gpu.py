"""Local Monte Carlo sweeps on the device (lq_metropolis_sweep, lq_heat_bath_sweep) against the
oracle's restatement of MetropolisHastingsSweep / HeatBathSweep
(src/simulation/monte_carlo/metropolis_hastings_sweep.rs, heat_bath.rs) in the same checkerboard
order with the same per-link Philox streams: FP64 links to 1e-12 of the largest entry, the same
number of accepted Metropolis updates and the same mean acceptance probability."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,L", [(2, 6), (3, 4), (4, 4)])
@pytest.mark.parametrize("start", ["random", "cold"])
def test_metropolis_matches_oracle(oracle_mod, lqgpu_mod, dim, L, start):
    O, G = oracle_mod, lqgpu_mod
    beta, n_update, spread, seed = 2.5, 2, 0.2, 41
    links = O.links_random(dim, L, O.Rng(8)) if start == "random" else O.links_cold(dim, L)
    ref = links
    with G.State(dim, L, 1.0, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        for sweep in range(2):
            ref, acc_ref, psum_ref = O.metropolis_sweep(dim, L, beta, ref, n_update, spread, seed, sweep)
            acc, pmean = s.metropolis_sweep(n_update, spread, seed, sweep)
            assert acc == acc_ref
            assert abs(pmean - psum_ref / (L ** dim * dim)) <= 1e-12
        got = s.link_matrix()
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("dim,L", [(2, 6), (3, 4), (4, 4)])
def test_heat_bath_matches_oracle(oracle_mod, lqgpu_mod, dim, L):
    O, G = oracle_mod, lqgpu_mod
    beta, seed = 3.0, 17
    ref = O.links_random(dim, L, O.Rng(9))
    with G.State(dim, L, 1.0, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(ref)
        for sweep in range(2):
            ref = O.heat_bath_sweep(dim, L, beta, ref, seed, sweep)
            s.heat_bath_sweep(seed, sweep)
        got = s.link_matrix()
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("dim,L", [(4, 2), (4, 6), (3, 6), (2, 10), (2, 34)])
def test_class_threads_cover_every_site_once(oracle_mod, lqgpu_mod, dim, L):
    """Classes that need several blocks of threads, rows of sites that cross 32-site tiles (L = 6, 10,
    34) and L = 2 (x + mu and x - mu coincide): a Metropolis then a heat-bath sweep, and an
    overrelaxation sweep from the random start, equal the oracle's, so the threads of a class update
    each of its links exactly once"""
    O, G = oracle_mod, lqgpu_mod
    beta = 2.5
    links = O.links_random(dim, L, O.Rng(12))
    with G.State(dim, L, 1.0, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        ref, acc_ref, _ = O.metropolis_sweep(dim, L, beta, links, 1, 0.2, 5, 0)
        acc, _ = s.metropolis_sweep(1, 0.2, 5, 0)
        assert acc == acc_ref
        ref = O.heat_bath_sweep(dim, L, beta, ref, 6, 0)
        s.heat_bath_sweep(6, 0)
        got = s.link_matrix()
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
        s.set_link_matrix(links)
        ref = O.overrelaxation_sweep(dim, L, links, 1)
        s.overrelaxation_sweep(G.OVERRELAX_REVERSE)
        got = s.link_matrix()
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_sweep_arguments(lqgpu_mod):
    G = lqgpu_mod
    with G.State(4, 3, 1.0, 2.0, G.PRECISION_F64) as s:  # odd L: no checkerboard
        with pytest.raises(G.LqError):
            s.metropolis_sweep(1, 0.1, 1, 0)
        with pytest.raises(G.LqError):
            s.heat_bath_sweep(1, 0)
    with G.State(4, 4, 1.0, 2.0, G.PRECISION_F64) as s:
        for n_update, spread in ((0, 0.1), (1, 0.0), (1, 1.0)):
            with pytest.raises(G.LqError):
                s.metropolis_sweep(n_update, spread, 1, 0)


@pytest.mark.parametrize("precision", [1, 2])
def test_fp32_forms_follow_fp64(oracle_mod, lqgpu_mod, precision):
    """The sweeps compute in double for every storage form; the FP32 forms differ by storage rounding."""
    O, G = oracle_mod, lqgpu_mod
    links = O.links_random(4, 4, O.Rng(2))
    out = []
    for p in (G.PRECISION_F64, precision):
        with G.State(4, 4, 1.0, 2.0, p) as s:
            s.set_link_matrix(links)
            s.metropolis_sweep(1, 0.1, 5, 0)
            out.append(s.link_matrix())
    tol = 1e-12 if precision == G.PRECISION_MIXED else 1e-6
    # a borderline accept decision could differ between storage forms; none does at this seed
    assert np.abs(out[1] - out[0]).max() <= tol
