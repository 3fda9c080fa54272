"""The algebra behind the FP64 state's projection and MD kernels, checked on the CPU with the oracle's
generators (the Gell-Mann basis T^a = lambda^a / 2 of src/su3.rs:24-194):

- the per-link transport table of k_adjoint_links: R_ab = 2 Re Tr(T^a U T^b U^dag),
  A_a = 2 Re Tr(T^a U U^dag), B_a = 2 Re Tr(T^a U^dag U), t = Tr(U U^dag), with a Hermitian X carried
  as x^a = 2 Re Tr(T^a X) and x^8 = Tr X, reproduces U X U^dag and U^dag X U for links that are not
  unitary (the leap-frog's first-order link update leaves them off the group);
- the symmetric constants of k_gauss_step_adj: 2 Re Tr(T^a X Y) = (1/2) d_acd x^c y^d for traceless
  Hermitian X, Y, with the table of d's nonzero entries the kernel uses;
- the four force parts of one plaquette in k_md_plaq equal the reference's staple form
  Im Tr(T^a U_mu(x) Sigma) term by term (src/simulation/state.rs:1420-1448).
"""
import itertools

import numpy as np
import pytest

S3 = np.sqrt(3.0)
# (1-based a, b, c): d_abc, as written in two_re_tr_generators_of_traceless_product
D_TABLE = {(1, 1, 8): 1 / S3, (2, 2, 8): 1 / S3, (3, 3, 8): 1 / S3, (8, 8, 8): -1 / S3,
           (4, 4, 8): -0.5 / S3, (5, 5, 8): -0.5 / S3, (6, 6, 8): -0.5 / S3, (7, 7, 8): -0.5 / S3,
           (1, 4, 6): 0.5, (1, 5, 7): 0.5, (2, 5, 6): 0.5, (3, 4, 4): 0.5, (3, 5, 5): 0.5,
           (2, 4, 7): -0.5, (3, 6, 6): -0.5, (3, 7, 7): -0.5}


@pytest.fixture(scope="module")
def gens(oracle_mod):
    return np.array([oracle_mod.to_complex(g) for g in oracle_mod.generators()])


def herm_components(T, X):
    """(x^0..x^7, x^8): 2 Re Tr(T^a X) and Tr X"""
    return np.concatenate([[2 * np.trace(T[a] @ X).real for a in range(8)], [np.trace(X).real]])


def from_components(T, x):
    return np.einsum("a,aij->ij", x[:8], T) + x[8] / 3.0 * np.eye(3)


def table(T, U):
    Ud = U.conj().T
    R = np.array([[2 * np.trace(T[a] @ U @ T[b] @ Ud).real for b in range(8)] for a in range(8)])
    A = np.array([2 * np.trace(T[a] @ U @ Ud).real for a in range(8)])
    B = np.array([2 * np.trace(T[a] @ Ud @ U).real for a in range(8)])
    t = np.trace(U @ Ud).real
    return R, A, B, t


def random_link(rng, off_group):
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3)))
    q = q / np.linalg.det(q) ** (1.0 / 3.0)
    return q * (1.0 + off_group * rng.normal(size=(3, 3)))


def random_hermitian(rng):
    h = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
    return h + h.conj().T


@pytest.mark.parametrize("off_group", [0.0, 1e-6, 1e-2])
def test_transport_table_reproduces_both_transports(gens, off_group):
    rng = np.random.default_rng(7)
    for _ in range(20):
        U = random_link(rng, off_group)
        X = random_hermitian(rng)
        R, A, B, t = table(gens, U)
        x = herm_components(gens, X)
        # U X U^dag: y^a = R_ab x^b + A_a x^8 / 3, y^8 = B_b x^b / 2 + t x^8 / 3
        fwd = np.concatenate([R @ x[:8] + A * x[8] / 3.0, [B @ x[:8] / 2.0 + t * x[8] / 3.0]])
        # U^dag X U: R^T and A, B swapped
        bwd = np.concatenate([R.T @ x[:8] + B * x[8] / 3.0, [A @ x[:8] / 2.0 + t * x[8] / 3.0]])
        assert np.allclose(from_components(gens, fwd), U @ X @ U.conj().T, atol=1e-12)
        assert np.allclose(from_components(gens, bwd), U.conj().T @ X @ U, atol=1e-12)


def test_traceless_components_lose_the_trace_off_the_group(gens):
    """Why the tables carry A, B and t: dropping the trace (8 components, R alone) is exact only on
    the group."""
    rng = np.random.default_rng(8)
    U = random_link(rng, 1e-3)
    E = np.einsum("a,aij->ij", rng.normal(size=8), gens)  # a traceless momentum
    assert abs(np.trace(U.conj().T @ E @ U)) > 1e-6


def test_symmetric_constants(gens):
    d = np.zeros((8, 8, 8))
    for a, b, c in itertools.product(range(8), repeat=3):
        d[a, b, c] = 2 * np.trace(gens[a] @ (gens[b] @ gens[c] + gens[c] @ gens[b])).real
    dt = np.zeros((8, 8, 8))
    for (a, b, c), v in D_TABLE.items():
        for p in set(itertools.permutations((a - 1, b - 1, c - 1))):
            dt[p] = v
    assert np.abs(d - dt).max() < 1e-15
    rng = np.random.default_rng(9)
    for _ in range(20):
        x, y = rng.normal(size=8), rng.normal(size=8)
        X, Y = np.einsum("a,aij->ij", x, gens), np.einsum("a,aij->ij", y, gens)
        want = np.array([2 * np.trace(gens[a] @ X @ Y).real for a in range(8)])
        assert np.allclose(0.5 * np.einsum("acd,c,d->a", dt, x, y), want, atol=1e-14)


def test_plaquette_force_parts_equal_the_staple_form(gens):
    """a = U_mu(x), b = U_nu(x+mu), c = U_mu(x+nu), d = U_nu(x); A = a b, B = d c.  The four parts
    k_md_plaq hands out equal Im Tr(T^a U S) with the reference's staples of each link."""
    rng = np.random.default_rng(10)
    im_tr = lambda M: np.array([np.trace(gens[k] @ M).imag for k in range(8)])
    dag = lambda M: M.conj().T
    for off_group in (0.0, 1e-3):
        a, b, c, d = (random_link(rng, off_group) for _ in range(4))
        A, B = a @ b, d @ c
        # (x, mu) with its +nu staple S = b c^dag d^dag; (x, nu) with its +mu staple c b^dag a^dag
        assert np.allclose(im_tr(A @ dag(B)), im_tr(a @ (b @ dag(c) @ dag(d))), atol=1e-13)
        assert np.allclose(-im_tr(A @ dag(B)), im_tr(d @ (c @ dag(b) @ dag(a))), atol=1e-13)
        # (x+nu, mu) with its -nu staple b^dag a^dag d; (x+mu, nu) with its -mu staple c^dag d^dag a
        assert np.allclose(im_tr(c @ dag(A) @ d), im_tr(c @ (dag(b) @ dag(a) @ d)), atol=1e-13)
        assert np.allclose(im_tr(b @ dag(B) @ a), im_tr(b @ (dag(c) @ dag(d) @ a)), atol=1e-13)
