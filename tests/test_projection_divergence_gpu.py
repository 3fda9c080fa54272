"""Large momenta (small beta) make the reference's Gauss projection diverge: its step is quadratic in
the Gauss law (src/field.rs:1301-1337) and the residual ends as NaN, where project_to_gauss returns
None and new_random_e_state panics (src/simulation/state.rs:1093-1108).  The device reports
LQ_ERR_GAUSS_PROJECTION for the oracle's diverging draw in every form, through the projection and the
HMC refresh, keeps the links and stays usable; in a batch the ensemble reports the status for each
trajectory, keeps its links, and the other ensembles run on."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIM, L = 4, 4


def draw(O, seed, std_dev):
    rng = O.Rng(seed)
    links = O.links_random(DIM, L, rng)
    return links, O.efield_normal(DIM, L, rng, std_dev)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_divergence_is_reported_like_the_oracle(oracle_mod, lqgpu_mod, precision):
    """beta 1/3, standard deviation 1.5: the oracle's residual is finite at the tests after 1, 5 and 9
    sweeps and NaN after 13 (the FP64 form matches that count; the FP32-arithmetic forms overflow no
    later)"""
    O, G = oracle_mod, lqgpu_mod
    links, e = draw(O, 100, 1.5)
    with G.State(DIM, L, 1000.0, 1.0 / 3.0, precision) as s:
        s.set_link_matrix(links)
        start = s.link_matrix()
        if precision == G.PRECISION_F64:
            for max_steps in (1, 5, 9):
                s.set_e_field(e)
                with pytest.raises(G.LqError) as err:
                    s.project_to_gauss(max_steps=max_steps)
                assert err.value.code == G.LQ_ERR_NOT_CONVERGED
        s.set_e_field(e)
        with pytest.raises(G.LqError) as err:
            s.project_to_gauss(max_steps=10001)
        assert err.value.code == G.LQ_ERR_GAUSS_PROJECTION
        with pytest.raises(G.LqError) as err:
            s.hmc_refresh_upload(e)
        assert err.value.code == G.LQ_ERR_GAUSS_PROJECTION
        assert np.array_equal(s.link_matrix(), start)
        # momenta of standard deviation 0.5 project on the same links afterwards
        s.set_e_field(O.efield_normal(DIM, L, O.Rng(7), 0.5))
        assert s.project_to_gauss(max_steps=10001) % 4 == 1


def test_batch_ensemble_whose_projection_diverges(lqgpu_mod):
    """beta 0.25 next to beta 2: the first ensemble fails every trajectory and keeps its links"""
    G = lqgpu_mod
    with G.Batch(DIM, [L, L], [1000.0, 1000.0], [0.25, 2.0], G.PRECISION_MIXED) as b:
        b.set_links_random(21)
        b.set_seed(5, 0)
        before = b.link_matrix(0)
        b.hmc_run(0.01, 4, 3, 10001)
        res = b.hmc_results()
        after = b.link_matrix(0)
    assert (res["status"][:, 0] == G.LQ_ERR_GAUSS_PROJECTION).all()
    assert not res["accepted"][:, 0].any()
    assert np.array_equal(before, after)
    assert (res["status"][:, 1] == 0).all()
