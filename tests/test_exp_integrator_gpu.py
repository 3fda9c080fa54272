"""The exponential link update U' = exp(i dt c E) U (LQ_SYMPLECTIC_EXP), by the Cayley-Hamilton
recursion of su3_exp_i (src/su3.rs:832-855).  The reference has no integrator that applies it,
so it is checked link by link against the oracle's restatement of su3_exp_i, for unitarity,
and for reversibility under a momentum flip (exact up to rounding on the group, O(dt^2) per
step for the reference's first-order update)."""
import numpy as np
import pytest

TOL = 1e-12


def fields(O, dim, L, seed, sd=0.5):
    rng = O.Rng(seed)
    return O.links_random(dim, L, rng), O.efield_normal(dim, L, rng, sd)


def unitarity_error(O, links):
    worst = 0.0
    for m18 in links:
        m = O.to_complex(m18)
        worst = max(worst, float(np.abs(m @ m.conj().T - np.eye(3)).max()))
    return worst


def test_oracle_exp_integrator_is_reversible_and_unitary(oracle_mod):
    O = oracle_mod
    dim, L, size, dt, n = 3, 3, 2.0, 0.05, 6
    links, e = fields(O, dim, L, 1)
    l1, e1 = O.integrate(dim, L, size, links, e, O.SYMPLECTIC_EXP, dt, n)
    assert unitarity_error(O, l1) < 1e-13
    l2, e2 = O.integrate(dim, L, size, l1, -e1, O.SYMPLECTIC_EXP, dt, n)
    assert np.abs(l2 - links).max() < 1e-12
    assert np.abs(-e2 - e).max() < 1e-12
    # the reference's first-order link update is not reversible at this order
    l1, e1 = O.integrate(dim, L, size, links, e, O.SYMPLECTIC, dt, n)
    l2, _ = O.integrate(dim, L, size, l1, -e1, O.SYMPLECTIC, dt, n)
    assert np.abs(l2 - links).max() > 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("dim,L", [(2, 4), (3, 3), (4, 3)])
@pytest.mark.parametrize("mode", [5, 6])
def test_exp_integrator_parity(oracle_mod, lqgpu_mod, dim, L, mode):
    O, G = oracle_mod, lqgpu_mod
    size, dt, n = 3.0, 0.04, 4
    links, e = fields(O, dim, L, 7)
    lr, er = O.integrate(dim, L, size, links, e, mode, dt, n)
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.integrate(mode, dt, n)
        assert np.abs(s.link_matrix() - lr).max() <= TOL
        assert np.abs(s.e_field() - er).max() <= TOL * max(1.0, np.abs(er).max())
        assert s.t == n


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-7), (2, 1e-5)])
def test_exp_integrator_reversible_on_device(oracle_mod, lqgpu_mod, precision, tol):
    """Forward n steps, flip the momenta, n steps, flip: back at the start.  Stated bounds per
    form: FP64 1e-12; mixed 1e-7 (its forces are FP32 products, relative error ~1e-7, on a
    momentum change of ~0.16 over the trajectory: ~1e-8 expected); f32 1e-5."""
    O, G = oracle_mod, lqgpu_mod
    dim, L, size, dt, n = 4, 4, 3.0, 0.02, 10
    links, e = fields(O, dim, L, 9)
    with G.State(dim, L, size, 1.0, precision) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.integrate(G.SYMPLECTIC_EXP, dt, n)
        s.set_e_field(-s.e_field())
        s.integrate(G.SYMPLECTIC_EXP, dt, n)
        du = np.abs(s.link_matrix() - links).max()
        de = np.abs(-s.e_field() - e).max()
        print("precision", precision, "reversibility error links", du, "E", de)
        assert du <= tol and de <= tol


@pytest.mark.gpu
def test_exp_link_update_stays_in_su3(oracle_mod, lqgpu_mod):
    O, G = oracle_mod, lqgpu_mod
    dim, L, size, dt = 4, 3, 1.0, 0.05
    links, e = fields(O, dim, L, 11)
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.integrate(G.SYMPLECTIC_EXP, dt, 40)
        exp_err = unitarity_error(O, s.link_matrix())
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.integrate(G.SYMPLECTIC, dt, 40)
        euler_err = unitarity_error(O, s.link_matrix())
    assert exp_err < 1e-13
    assert euler_err > 1e-6  # the first-order update leaves the group


@pytest.mark.gpu
def test_hmc_with_exp_link_update(lqgpu_mod):
    """HMC proposals with the exponential update: |dH| small and acceptance high at size 1000."""
    G = lqgpu_mod
    with G.State(4, 6, 1000.0, 1.0, G.PRECISION_MIXED) as s:
        s.set_links_random(3)
        s.set_link_update(G.LINK_UPDATE_EXP)
        for k in range(4):
            r = s.hmc_trajectory(0.01, 10, 5, k, 0.5)
            assert abs(r["delta_h"]) < 1e-3 and r["accepted"]
