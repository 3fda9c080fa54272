"""lq_leapfrog_adjoint on the device: the reverse-mode adjoint of a symplectic leap-frog
trajectory for O = Re average_trace_plaquette(U_n) / 3.

* parity: the CUDA adjoint against the numpy restatement of the same recursion
  (tests/adjoint_ref.py, itself checked against central differences on the CPU), FP64, 1e-12;
* the differentiation configuration: D = 4, 16^4, beta 2, random links (seed 2), size 1,
  momenta N(0, 0.5/beta), 50 steps of dt 0.01: dO/dbeta for momenta E0 beta0 / beta against
  the central difference in beta with delta beta = 1e-4, relative tolerance 1e-6 (the
  difference quotient's truncation is O(delta beta^2) ~ 1e-8 relative, its rounding ~1e-11);
* the result does not depend on the checkpoint interval (bitwise: the segments are recomputed
  by the forward pass's own launches);
* FP32: the adjoint of the FP32 form against FP64 at 16^4, relative 1e-3."""
import numpy as np
import pytest

import adjoint_ref as A

pytestmark = pytest.mark.gpu


def test_adjoint_matches_numpy_recursion(oracle_mod, lqgpu_mod):
    O, G = oracle_mod, lqgpu_mod
    dim, L, size, dt, n, beta = 3, 3, 1.0, 0.02, 5, 2.0
    rng = O.Rng(4)
    links = O.links_random(dim, L, rng)
    e0 = O.efield_normal(dim, L, rng, 0.5 / beta)
    obj, lam_u, lam_e = A.leapfrog_adjoint(O, dim, L, size, links, e0, dt, n)
    with G.State(dim, L, size, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e0)
        r = s.leapfrog_adjoint(dt, n, checkpoint_every=2)
        assert np.array_equal(s.link_matrix(), links)  # the state is left unchanged
    assert abs(r["objective"] - obj) <= 1e-14
    gu = np.array([O.to_complex(m) for m in r["grad_links"]]).reshape(lam_u.shape)
    scale = np.abs(lam_u).max()
    assert np.abs(gu - lam_u).max() <= 1e-12 * scale
    assert np.abs(r["grad_efield"] - lam_e.reshape(r["grad_efield"].shape)).max() <= 1e-12 * np.abs(lam_e).max()
    assert abs(r["d_objective_d_beta"] + np.sum(lam_e.reshape(e0.shape) * e0) / beta) <= 1e-12 * scale


def _objective(G, s, links, e, dt, n):
    s.set_link_matrix(links)
    s.set_e_field(e)
    s.integrate(G.SYMPLECTIC, dt, n)
    return s.average_trace_plaquette().real / 3.0


def test_dplaq_dbeta_against_finite_difference_16x4(lqgpu_mod):
    G = lqgpu_mod
    dim, L, size, beta, dt, n, db = 4, 16, 1.0, 2.0, 0.01, 50, 1e-4
    with G.State(dim, L, size, beta, G.PRECISION_F64) as s:
        s.set_links_random(2)
        s.set_e_field(np.random.default_rng(2).normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8)))
        links, e0 = s.link_matrix(), s.e_field()
        r = s.leapfrog_adjoint(dt, n, grads=False)
        op = _objective(G, s, links, e0 * beta / (beta + db), dt, n)
        om = _objective(G, s, links, e0 * beta / (beta - db), dt, n)
        o0 = _objective(G, s, links, e0, dt, n)
    fd = (op - om) / (2 * db)
    print("16^4 FP64: O", r["objective"], "dO/dbeta adjoint", r["d_objective_d_beta"], "central difference", fd,
          "work bytes", r["work_bytes"])
    assert abs(r["objective"] - o0) <= 1e-13
    assert abs(r["d_objective_d_beta"] - fd) <= 1e-6 * abs(fd)


def test_checkpoint_interval_does_not_change_the_result(lqgpu_mod):
    G = lqgpu_mod
    with G.State(4, 4, 1.0, 2.0, G.PRECISION_F64) as s:
        s.set_links_random(7)
        s.set_e_field(np.random.default_rng(7).normal(0.0, 0.25, size=(4 ** 4, 4, 8)))
        runs = [s.leapfrog_adjoint(0.01, 12, checkpoint_every=c) for c in (0, 1, 5, 12)]
    for r in runs[1:]:
        assert r["d_objective_d_beta"] == runs[0]["d_objective_d_beta"]
        assert np.array_equal(r["grad_links"], runs[0]["grad_links"])
        assert np.array_equal(r["grad_efield"], runs[0]["grad_efield"])
    assert runs[3]["work_bytes"] > runs[0]["work_bytes"]  # one segment holds every step


@pytest.mark.parametrize("precision", [2, 1])
def test_fp32_adjoint_against_fp64(lqgpu_mod, precision):
    G = lqgpu_mod
    dim, L, beta = 4, 16, 2.0
    out = []
    for p in (G.PRECISION_F64, precision):
        with G.State(dim, L, 1.0, beta, p) as s:
            s.set_links_random(2)
            s.set_e_field(np.random.default_rng(2).normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8)))
            out.append(s.leapfrog_adjoint(0.01, 50, grads=False))
    rel = abs(out[1]["d_objective_d_beta"] - out[0]["d_objective_d_beta"]) / abs(out[0]["d_objective_d_beta"])
    print("precision", precision, "dO/dbeta", out[1]["d_objective_d_beta"], "FP64", out[0]["d_objective_d_beta"],
          "relative difference", rel)
    assert rel <= 1e-3
    assert abs(out[1]["objective"] - out[0]["objective"]) <= 1e-5
