"""The Gauss projection as one CUDA graph launch (a conditional while node driven by a device-side
convergence test) against the host-driven loop (one host read of the residual per test): the same
number of sweeps, bitwise the same projected field and Gauss law, the same errors at the step limit
and on a non-finite field, and the same trajectories while the graph cache meets every link buffer
and E/G buffer order of a state.  Every form: the FP32-arithmetic ones sweep with one fused kernel on
double-buffered fields, the FP64 one with its step and Gauss-law kernels in place."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIM, L, SIZE, BETA = 4, 6, 1000.0, 2.0


def pair(G, precision, seed=3):
    a = G.State(DIM, L, SIZE, BETA, precision)
    b = G.State(DIM, L, SIZE, BETA, precision)
    a.set_links_random(seed)
    b.set_link_matrix(a.link_matrix())
    b.set_projection_graph(False)
    return a, b


@pytest.mark.parametrize("precision", [1, 2, 0])
def test_projection_graph_equals_host_loop(lqgpu_mod, precision):
    G = lqgpu_mod
    a, b = pair(G, precision)
    rng = np.random.default_rng(5)
    with a, b:
        for k in range(5):
            e_raw = rng.normal(0.0, 0.5 / BETA, size=(L ** DIM, DIM, 8))
            sa, sb = a.hmc_refresh_upload(e_raw), b.hmc_refresh_upload(e_raw)
            assert sa == sb and sa % 4 == 1
            assert np.array_equal(a.e_field(), b.e_field())
            assert np.array_equal(a.gauss(), b.gauss())
            assert a.gauss_sum_div() == b.gauss_sum_div()
            # alternate accept / reject so the link buffer of the state rotates both ways
            pa, _, _ = a.hmc_propose(0.01, 4)
            pb, _, _ = b.hmc_propose(0.01, 4)
            assert pa == pb
            a.hmc_decide(k % 2 == 0)
            b.hmc_decide(k % 2 == 0)
            assert np.array_equal(a.link_matrix(), b.link_matrix())


@pytest.mark.parametrize("precision", [1, 2, 0])
def test_projection_graph_trajectories(lqgpu_mod, precision):
    G = lqgpu_mod
    a, b = pair(G, precision, seed=8)
    with a, b:
        for k in range(6):
            u = 0.5 if k % 3 else 0.999999
            ra = a.hmc_trajectory(0.01, 5, 21, k, u)
            rb = b.hmc_trajectory(0.01, 5, 21, k, u)
            assert ra == rb
        assert np.array_equal(a.link_matrix(), b.link_matrix())
        assert np.array_equal(a.e_field(), b.e_field())


@pytest.mark.parametrize("precision", [1, 2, 0])
def test_projection_graph_errors(lqgpu_mod, precision):
    G = lqgpu_mod
    a, b = pair(G, precision)
    rng = np.random.default_rng(6)
    e_raw = rng.normal(0.0, 0.5 / BETA, size=(L ** DIM, DIM, 8))
    with a, b:
        # a random draw is not projected after one sweep: both stop at the limit
        codes = []
        for s in (a, b):
            s.set_e_field(e_raw)
            with pytest.raises(G.LqError) as err:
                s.project_to_gauss(max_steps=2)
            codes.append(err.value.code)
        assert codes == [G.LQ_ERR_NOT_CONVERGED] * 2
        assert np.array_equal(a.e_field(), b.e_field())
        # a non-finite momentum: the residual is NaN at the first test
        bad = e_raw.copy()
        bad[7, 1, 3] = np.nan
        codes = []
        for s in (a, b):
            s.set_e_field(bad)
            with pytest.raises(G.LqError) as err:
                s.project_to_gauss()
            codes.append(err.value.code)
        assert codes == [G.LQ_ERR_GAUSS_PROJECTION] * 2
        # the state stays usable: a finite field projects again, with the same result
        for s in (a, b):
            s.set_e_field(e_raw)
        assert a.project_to_gauss() == b.project_to_gauss()
        assert np.array_equal(a.e_field(), b.e_field())


@pytest.mark.parametrize("precision", [1, 2, 0])
def test_projection_graph_without_step_limit(lqgpu_mod, precision):
    """max_steps <= 0: the host loop has no limit, the graph its own bound; a field that converges
    gives the same sweeps and field either way."""
    G = lqgpu_mod
    a, b = pair(G, precision, seed=4)
    e_raw = np.random.default_rng(9).normal(0.0, 0.5 / BETA, size=(L ** DIM, DIM, 8))
    with a, b:
        for s in (a, b):
            s.set_e_field(e_raw)
        assert a.project_to_gauss(max_steps=0) == b.project_to_gauss(max_steps=0)
        assert np.array_equal(a.e_field(), b.e_field())


@pytest.mark.parametrize("dim,Lt", [(2, 2), (2, 3), (3, 2), (3, 3), (4, 2), (4, 3)])
def test_projection_graph_tiny_lattices(lqgpu_mod, dim, Lt):
    """L = 2 (x + mu and x - mu coincide) and volumes that end inside a tile, D = 2, 3, 4: trajectories
    with the graph equal those with the host loop."""
    G = lqgpu_mod
    a = G.State(dim, Lt, SIZE, BETA, G.PRECISION_MIXED)
    b = G.State(dim, Lt, SIZE, BETA, G.PRECISION_MIXED)
    with a, b:
        a.set_links_random(7)
        b.set_link_matrix(a.link_matrix())
        b.set_projection_graph(False)
        for k in range(3):
            assert a.hmc_trajectory(0.01, 4, 3, k, 0.5) == b.hmc_trajectory(0.01, 4, 3, k, 0.5)
        assert np.array_equal(a.link_matrix(), b.link_matrix())


@pytest.mark.parametrize("precision", [1, 0])
def test_projection_graph_profile_counts(lqgpu_mod, precision):
    """The graph's profile slot counts the Gauss law, every sweep and every test (FP64: the transport
    tables, the first Gauss law, then a step and a Gauss law per sweep)."""
    G = lqgpu_mod
    with G.State(DIM, L, SIZE, BETA, precision) as s:
        s.set_links_random(2)
        s.set_e_field_normal(4, 0, 0.25)
        s.profile_enable(True)
        s.profile_read(reset=True)
        steps = s.project_to_gauss()
        prof = s.profile_read(reset=True)
        kernels = 1 + steps if precision else 2 + 2 * steps
        assert prof["gauss_sweep"][0] == kernels + (steps + 3) // 4
        assert prof["gauss_sweep"][1] > 0.0
