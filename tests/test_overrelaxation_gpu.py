"""Overrelaxation sweeps on the device (lq_overrelaxation_sweep: OverrelaxationSweepRotation and
OverrelaxationSweepReverse, src/simulation/monte_carlo/overrelaxation.rs) against the oracle's
restatement in the same checkerboard order: FP64 links to 1e-12 of the largest entry; the link
Hamiltonian conserved in every form (the reference's same_energy tests); the reference's documented
use, heat bath and overrelaxation alternating from a cold start, step for step with the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("dim,L", [(2, 6), (3, 4), (4, 4)])
@pytest.mark.parametrize("start", ["random", "cold"])
def test_overrelaxation_matches_oracle(oracle_mod, lqgpu_mod, method, dim, L, start):
    O, G = oracle_mod, lqgpu_mod
    links = O.links_random(dim, L, O.Rng(30 + dim)) if start == "random" else O.links_cold(dim, L)
    ref = links
    with G.State(dim, L, 1.0, 2.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        for _ in range(2):
            ref = O.overrelaxation_sweep(dim, L, ref, method)
            s.overrelaxation_sweep(method)
        got = s.link_matrix()
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-7), (2, 1e-5)])
def test_overrelaxation_conserves_the_link_hamiltonian(lqgpu_mod, method, precision, tol):
    """FP64 to 1e-12 relative; the FP32-arithmetic forms sum the link Hamiltonian from FP32 traces of
    the hi parts, which bounds what they can show (mixed 1e-7, f32 1e-5)."""
    G = lqgpu_mod
    with G.State(4, 6, 1.0, 2.0, precision) as s:
        s.set_links_random(5)
        for _ in range(3):
            h = s.hamiltonian_links()
            s.overrelaxation_sweep(method)
            h2 = s.hamiltonian_links()
            assert abs(h2 - h) <= tol * abs(h)


def test_heat_bath_and_overrelaxation_alternating(oracle_mod, lqgpu_mod):
    """The reference's documented use (overrelaxation.rs module example): LatticeStateDefault<3>,
    cold start, beta 8, 4 points; heat bath then overrelaxation (reverse), twice."""
    O, G = oracle_mod, lqgpu_mod
    dim, L, beta, seed = 3, 4, 8.0, 7
    ref = O.links_cold(dim, L)
    with G.State(dim, L, 1.0, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(ref)
        for k in range(2):
            ref = O.heat_bath_sweep(dim, L, beta, ref, seed, k)
            s.heat_bath_sweep(seed, k)
            ref = O.overrelaxation_sweep(dim, L, ref, 1)
            s.overrelaxation_sweep(G.OVERRELAX_REVERSE)
        got = s.link_matrix()
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_overrelaxation_arguments(lqgpu_mod):
    G = lqgpu_mod
    with G.State(4, 3, 1.0, 2.0, G.PRECISION_F64) as s:
        with pytest.raises(G.LqError) as err:
            s.overrelaxation_sweep(G.OVERRELAX_ROTATION)
        assert err.value.code == G.LQ_ERR_INVALID_ARGUMENT
    with G.State(4, 4, 1.0, 2.0, G.PRECISION_F64) as s:
        with pytest.raises(G.LqError) as err:
            s.overrelaxation_sweep(2)
        assert err.value.code == G.LQ_ERR_INVALID_ARGUMENT
