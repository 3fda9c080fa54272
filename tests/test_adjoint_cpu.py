"""The leap-frog adjoint's recursion (tests/adjoint_ref.py, the formulas of csrc/adjoint.cuh)
against central differences of the oracle's symplectic integrator (the reference's
integrate_symplectic restated): along a random momentum direction, along single-link
rotations exp(i eps T^a) U, and in beta for momenta E0 beta0 / beta."""
import numpy as np

import adjoint_ref as A


def test_adjoint_recursion_matches_central_differences(oracle_mod):
    O = oracle_mod
    dim, L, size, dt, n, beta, eps = 3, 3, 1.0, 0.02, 5, 2.0, 1e-6
    rng = O.Rng(4)
    links = O.links_random(dim, L, rng)
    e0 = O.efield_normal(dim, L, rng, 0.5 / beta)
    obj, lam_u, lam_e = A.leapfrog_adjoint(O, dim, L, size, links, e0, dt, n)
    assert abs(obj - A.objective(O, dim, L, size, links, e0, dt, n)) < 1e-15

    def o(lk, e):
        return A.objective(O, dim, L, size, lk, e, dt, n)

    v = np.random.default_rng(0).normal(size=e0.shape)
    fd = (o(links, e0 + eps * v) - o(links, e0 - eps * v)) / (2 * eps)
    assert abs(fd - np.sum(lam_e.reshape(v.shape) * v)) < 1e-9
    db = 1e-4
    fdb = (o(links, e0 * beta / (beta + db)) - o(links, e0 * beta / (beta - db))) / (2 * db)
    adj_b = -np.sum(lam_e.reshape(e0.shape) * e0) / beta
    assert abs(fdb - adj_b) < 1e-8 * max(1e-3, abs(adj_b)) + 1e-11
    T = A.generators(O)
    U = A.to_mats(O, links, dim, L)
    for x, mu, a in [(0, 0, 0), (5, 1, 3), (13, 2, 7), (20, 0, 5)]:
        w, vec = np.linalg.eigh(T[a])
        def rot(s):
            Uc = U.copy()
            Uc[x, mu] = (vec @ np.diag(np.exp(1j * s * eps * w)) @ vec.conj().T) @ Uc[x, mu]
            return o(A.from_mats(O, Uc), e0)
        fdl = (rot(1) - rot(-1)) / (2 * eps)
        adj = np.real(np.trace(lam_u[x, mu].conj().T @ (1j * T[a] @ U[x, mu])))
        assert abs(fdl - adj) < 1e-9
