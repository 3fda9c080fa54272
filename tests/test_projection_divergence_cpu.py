"""The reference's Gauss projection step (EField::project_to_gauss_step, src/field.rs:1301-1337) is
quadratic in the Gauss law: e'^a = 2 Re Tr(T^a [(u G(x) u^dag G(x+mu) - G(x)) K + T^a e^a]).  It
contracts for small G and diverges for large momenta, until the residual is NaN and
project_to_gauss returns None (src/field.rs:1282-1284), on which new_random_e_state panics
(src/simulation/state.rs:1093-1108).  The momenta's standard deviation is 0.5 / beta, so this happens
at small beta: in the oracle, a 4^4 lattice with random links fails for 1 of 6 draws at beta 0.5 and for
every draw at beta 1/3.  These cases pin the failure the device reports as LQ_ERR_GAUSS_PROJECTION."""
import pytest

DIM, L = 4, 4


def draw(O, seed, std_dev):
    rng = O.Rng(seed)
    links = O.links_random(DIM, L, rng)
    return links, O.efield_normal(DIM, L, rng, std_dev)


def test_projection_diverges_to_nan_for_large_momenta(oracle_mod):
    """beta = 1/3 (standard deviation 1.5): the residual grows from 1.2e3 and is NaN at the fourth test
    (after 13 sweeps); the tests after 1, 5 and 9 sweeps still see a finite residual"""
    O = oracle_mod
    links, e = draw(O, 100, 1.5)
    assert 1e3 < O.gauss_sum_div(DIM, L, links, e) < 2e3
    for max_steps in (1, 5, 9):
        with pytest.raises(O.OracleError, match="status 10"):
            O.project_to_gauss(DIM, L, links, e, max_steps)
    with pytest.raises(O.OracleError, match="status 7"):
        O.project_to_gauss(DIM, L, links, e, 10001)


@pytest.mark.parametrize("seed", range(100, 104))
def test_every_draw_diverges_at_beta_one_third(oracle_mod, seed):
    O = oracle_mod
    links, e = draw(O, seed, 1.5)
    with pytest.raises(O.OracleError, match="status 7"):
        O.project_to_gauss(DIM, L, links, e, 10001)


def test_the_same_links_project_at_beta_one(oracle_mod):
    """the links of the diverging case with momenta of standard deviation 0.5 (beta 1) converge"""
    O = oracle_mod
    links, _ = draw(O, 100, 1.5)
    e = O.efield_normal(DIM, L, O.Rng(7), 0.5)
    projected, steps = O.project_to_gauss(DIM, L, links, e, 10001)
    assert steps % 4 == 1
    assert O.gauss_sum_div(DIM, L, links, projected) <= 2.220446049250313e-16 * L ** DIM * 320
