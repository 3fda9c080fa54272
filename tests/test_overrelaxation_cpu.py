"""The oracle's restatement of OverrelaxationSweepRotation / OverrelaxationSweepReverse
(src/simulation/monte_carlo/overrelaxation.rs), pinned three ways:

* per link against LAPACK's SVD (numpy): the reference takes nalgebra's SVD of a = staple^dag, and
  for distinct singular values both updates are independent of which SVD computes U and V;
* per link, each update is an involution for a fixed staple (rotation: rot (rot U^dag rot)^dag rot = U;
  reverse: reverse(reverse(X)) = X);
* per sweep, the reference's own test (same_energy_rotation / same_energy_reverse,
  overrelaxation.rs:220-262): the link Hamiltonian is conserved, D = 3, L = 4, beta 1."""
import numpy as np
import pytest


def random_complex(rng, n=3):
    return rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))


def reverse(x):
    r = -x.copy()
    np.fill_diagonal(r, np.diag(x))
    return r


def svd_update(link, staple, method):
    u, _, vh = np.linalg.svd(staple.conj().T)
    if method == 0:
        rot = u @ vh
        return rot @ link.conj().T @ rot
    return u @ reverse(u.conj().T @ link @ vh.conj().T) @ vh


@pytest.mark.parametrize("method", [0, 1])
def test_link_update_matches_lapack_svd(oracle_mod, method):
    O = oracle_mod
    rng = np.random.default_rng(11 + method)
    worst = 0.0
    for _ in range(200):
        link = np.linalg.qr(random_complex(rng))[0]  # unitary
        staple = random_complex(rng) * 2.0
        got = O.to_complex(O.overrelax_link(O.from_complex(link), O.from_complex(staple), method))
        want = svd_update(link, staple, method)
        worst = max(worst, np.abs(got - want).max())
    assert worst <= 1e-12, worst


@pytest.mark.parametrize("eps", [1e-2, 1e-5, 1e-9, 0.0])
def test_rotation_matches_lapack_on_near_degenerate_staples(oracle_mod, eps):
    """Staples 6 W + eps X (W in SU(3)) have singular values eps apart, the slowest case for the
    fixed number of Jacobi sweeps; the rotation's polar factor stays unique down to eps = 0."""
    O = oracle_mod
    rng = np.random.default_rng(31)
    worst = 0.0
    for _ in range(200):
        link = np.linalg.qr(random_complex(rng))[0]
        w = np.linalg.qr(random_complex(rng))[0]
        staple = 6.0 * w / np.linalg.det(w) ** (1.0 / 3.0) + eps * random_complex(rng)
        got = O.to_complex(O.overrelax_link(O.from_complex(link), O.from_complex(staple), 0))
        worst = max(worst, np.abs(got - svd_update(link, staple, 0)).max())
    assert worst <= 1e-12, worst


@pytest.mark.parametrize("method", [0, 1])
def test_link_update_is_an_involution(oracle_mod, method):
    O = oracle_mod
    rng = np.random.default_rng(21 + method)
    for _ in range(50):
        link = O.from_complex(np.linalg.qr(random_complex(rng))[0])
        staple = O.from_complex(random_complex(rng))
        twice = O.overrelax_link(O.overrelax_link(link, staple, method), staple, method)
        assert np.abs(twice - link).max() <= 1e-12


@pytest.mark.parametrize("method", [0, 1])
def test_sweep_conserves_the_link_hamiltonian(oracle_mod, method):
    """same_energy_rotation / same_energy_reverse: |h - h2| < eps 100 4^3 (h + h2) / 2 on D = 3, L = 4,
    beta 1, ten random starts"""
    O = oracle_mod
    rng = O.Rng(0x457893F44AB067F0)
    dim, L, beta = 3, 4, 1.0
    for _ in range(10):
        links = O.links_random(dim, L, rng)
        h = O.hamiltonian_links(dim, L, beta, links)
        h2 = O.hamiltonian_links(dim, L, beta, O.overrelaxation_sweep(dim, L, links, method))
        assert abs(h - h2) < 2.220446049250313e-16 * 100 * 4 ** 3 * (h + h2) * 0.5


def test_sweep_rejects_odd_lattices_and_unknown_methods(oracle_mod):
    O = oracle_mod
    links = O.links_random(3, 3, O.Rng(1))
    with pytest.raises(O.OracleError):
        O.overrelaxation_sweep(3, 3, links, 0)
    links = O.links_random(3, 4, O.Rng(1))
    with pytest.raises(O.OracleError):
        O.overrelaxation_sweep(3, 4, links, 2)
