"""The gauge force as the backward of the Wilson action (lq_wilson_action /
lq_wilson_action_backward): against the reference's force (derivative_e,
src/simulation/state.rs:1420-1448, through the oracle) and against central finite differences
of the action along all 8 generators.

Finite-difference configuration (the differentiation workload): D = 4, 16^4, beta 2,
random links (seed 2), FP64, eps = 1e-5, 1024 random links x 8 generators.  The action is a sum
of ~4e5 plaquette terms, so S itself carries ~1e-10 of rounding; the difference quotient is
therefore compared with a 1e-4 absolute tolerance (the gradient entries are O(1)).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,L", [(2, 5), (3, 4), (4, 3)])
def test_backward_is_the_reference_force(oracle_mod, lqgpu_mod, dim, L):
    O, G = oracle_mod, lqgpu_mod
    size, beta = 7.0, 2.5
    rng = O.Rng(31)
    links = O.links_random(dim, L, rng)
    f_ref = O.derivative_e(dim, L, size, links)
    with G.State(dim, L, size, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        grad = s.wilson_action_backward()
        assert abs(s.wilson_action() - O.hamiltonian_links(dim, L, beta, links)) <= 1e-12 * s.wilson_action()
    f = -math.sqrt(6.0) / (size * beta) * grad
    assert np.abs(f - f_ref).max() <= 1e-12 * max(1.0, np.abs(f_ref).max())


def test_backward_against_central_differences(lqgpu_mod):
    G = lqgpu_mod
    dim, L, beta, eps = 4, 16, 2.0, 1e-5
    rng = np.random.default_rng(2)
    with G.State(dim, L, 1.0, beta, G.PRECISION_F64) as s:
        s.set_links_random(2)
        grad = s.wilson_action_backward().reshape(-1, 8)
        links = rng.choice(L ** dim * dim, size=1024, replace=False)
        worst = 0.0
        for link in links:
            for a in range(8):
                s.link_rotate(int(link), a, eps)
                sp = s.wilson_action()
                s.link_rotate(int(link), a, -2 * eps)
                sm = s.wilson_action()
                s.link_rotate(int(link), a, eps)
                fd = (sp - sm) / (2 * eps)
                worst = max(worst, abs(fd - grad[link, a]))
        print("max |central difference - backward| over 1024 links x 8 generators:", worst)
        assert worst <= 1e-4
        assert np.abs(grad).max() > 0.1


@pytest.mark.parametrize("precision,tol", [(1, 1e-5), (2, 1e-5)])
def test_backward_in_fp32_forms(oracle_mod, lqgpu_mod, precision, tol):
    O, G = oracle_mod, lqgpu_mod
    dim, L = 4, 4
    links = O.links_random(dim, L, O.Rng(5))
    out = []
    for p in (G.PRECISION_F64, precision):
        with G.State(dim, L, 1.0, 2.0, p) as s:
            s.set_link_matrix(links)
            out.append(s.wilson_action_backward())
    assert np.abs(out[1] - out[0]).max() <= tol * np.abs(out[0]).max()
