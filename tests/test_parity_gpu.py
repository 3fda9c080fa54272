"""FP64 parity of the CUDA library with the CPU oracle, through the C ABI.

Both sides get the same inputs (links, momenta and accept uniforms drawn by the oracle's
seeded Xoshiro256++).  Tolerance of the FP64 form: 1e-12, relative to max(1, |value|) per
link / coefficient, and 1e-12 * |H| for Hamiltonians and Delta H (the reference's own
Hamiltonian sums are order-nondeterministic at the 1e-16 * |H| level).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(1.0, float(np.abs(b).max())))


def gen_coeffs(O, m18):
    """g^a = 2 Re Tr(T^a G) of a 3x3 complex matrix (serde layout)."""
    G = O.to_complex(m18)
    return np.array([2 * np.trace(O.to_complex(t) @ G).real for t in O.generators()])


def random_fields(O, dim, L, seed, e_sd=0.5):
    rng = O.Rng(seed)
    links = O.links_random(dim, L, rng)
    e = O.efield_normal(dim, L, rng, e_sd)
    return links, e


CASES = [(2, 4), (2, 5), (3, 4), (3, 3), (4, 3), (4, 4)]


@pytest.mark.parametrize("dim,L", CASES)
def test_upload_download_roundtrip(oracle_mod, lqgpu_mod, dim, L):
    O, G = oracle_mod, lqgpu_mod
    links, e = random_fields(O, dim, L, 11)
    with G.State(dim, L, 1000.0, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        assert np.array_equal(s.link_matrix(), links)
        assert np.array_equal(s.e_field(), e)


@pytest.mark.parametrize("dim,L", CASES)
def test_observables(oracle_mod, lqgpu_mod, dim, L):
    O, G = oracle_mod, lqgpu_mod
    beta = 2.0
    links, e = random_fields(O, dim, L, 100 + dim * 10 + L)
    with G.State(dim, L, 1000.0, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        hu_ref = O.hamiltonian_links(dim, L, beta, links)
        he_ref = O.hamiltonian_efield(dim, L, beta, e)
        assert abs(s.hamiltonian_links() - hu_ref) <= TOL * abs(hu_ref)
        assert abs(s.hamiltonian_efield() - he_ref) <= TOL * abs(he_ref)
        assert abs(s.hamiltonian_total() - (hu_ref + he_ref)) <= TOL * abs(hu_ref + he_ref)
        p = s.average_trace_plaquette()
        p_ref = O.average_trace_plaquette(dim, L, links)
        assert abs(p - p_ref) <= TOL
        g = s.gauss()
        g_ref = np.stack([gen_coeffs(O, O.gauss(dim, L, links, e, x)) for x in range(L ** dim)])
        assert rel(g, g_ref) <= TOL
        gsd_ref = O.gauss_sum_div(dim, L, links, e)
        assert abs(s.gauss_sum_div() - gsd_ref) <= TOL * max(1.0, gsd_ref)


def test_cold_state_values(lqgpu_mod):
    G = lqgpu_mod
    with G.State(4, 4, 1.0, 3.0, G.PRECISION_F64) as s:
        assert s.hamiltonian_links() == 0.0
        assert s.hamiltonian_efield() == 0.0
        assert s.average_trace_plaquette() == 3.0 + 0.0j
        assert s.gauss_sum_div() == 0.0


def test_sim_cold(lqgpu_mod):
    """test_sim_cold (src/test/mod.rs:430-453): a cold state is bit-exactly unchanged."""
    G = lqgpu_mod
    with G.State(4, 4, 10.0, 0.1, G.PRECISION_F64) as s:
        u0, e0 = s.link_matrix(), s.e_field()
        s.integrate(G.SYNC_LEAP, 0.1)
        assert np.array_equal(s.link_matrix(), u0) and np.array_equal(s.e_field(), e0)
        s.integrate(G.LEAP_LEAP, 0.1)
        assert np.array_equal(s.link_matrix(), u0) and np.array_equal(s.e_field(), e0)
        s.integrate(G.LEAP_SYNC, 0.1)
        assert np.array_equal(s.link_matrix(), u0) and np.array_equal(s.e_field(), e0)
        assert s.t == 2


@pytest.mark.parametrize("dim,L", [(2, 4), (3, 3), (4, 3)])
@pytest.mark.parametrize("mode,n", [(4, 1), (4, 3), (0, 1), (0, 2)])
def test_integrate_sync_modes(oracle_mod, lqgpu_mod, dim, L, mode, n):
    O, G = oracle_mod, lqgpu_mod
    size, dt = 7.0, 0.05
    links, e = random_fields(O, dim, L, 3)
    lr, er = O.integrate(dim, L, size, links, e, mode, dt, n)
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.integrate(mode, dt, n)
        assert rel(s.link_matrix(), lr) <= TOL
        assert rel(s.e_field(), er) <= TOL
        assert s.t == n


@pytest.mark.parametrize("dim", [2, 3, 4])
@pytest.mark.parametrize("mode,n", [(4, 3), (0, 2)])
def test_smallest_lattice_wraps(oracle_mod, lqgpu_mod, dim, mode, n):
    """L = 2: x + mu and x - mu are the same site, so each plaquette meets the wrap-around in all its
    links, and the FP64 MD step's force parts for a link arrive from a site that is both its forward
    and its backward neighbour; the projection on the same fields too."""
    O, G = oracle_mod, lqgpu_mod
    size, dt, L = 7.0, 0.05, 2
    links, e = random_fields(O, dim, L, 31)
    lr, er = O.integrate(dim, L, size, links, e, mode, dt, n)
    e_ref, steps_ref = O.project_to_gauss(dim, L, links, e)
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.integrate(mode, dt, n)
        assert rel(s.link_matrix(), lr) <= TOL
        assert rel(s.e_field(), er) <= TOL
        s.set_link_matrix(links)
        s.set_e_field(e)
        assert s.project_to_gauss() == steps_ref
        assert rel(s.e_field(), e_ref) <= TOL


@pytest.mark.parametrize("dim,L", [(2, 4), (3, 3), (4, 3)])
def test_leapfrog_chain(oracle_mod, lqgpu_mod, dim, L):
    """sync_leap, leap_leap x2, leap_sync and simulate_using_leapfrog_n"""
    O, G = oracle_mod, lqgpu_mod
    size, dt = 3.0, 0.02
    links, e = random_fields(O, dim, L, 5)
    l1, e1 = O.integrate(dim, L, size, links, e, O.SYNC_LEAP, dt, 1)
    l2, e2 = O.integrate(dim, L, size, l1, e1, O.LEAP_LEAP, dt, 2)
    l3, e3 = O.integrate(dim, L, size, l2, e2, O.LEAP_SYNC, dt, 1)
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.integrate(G.SYNC_LEAP, dt)
        assert s.info()["is_leap"]
        assert rel(s.e_field(), e1) <= TOL
        s.integrate(G.LEAP_LEAP, dt, 2)
        assert rel(s.link_matrix(), l2) <= TOL and rel(s.e_field(), e2) <= TOL
        s.integrate(G.LEAP_SYNC, dt)
        assert not s.info()["is_leap"]
        assert rel(s.link_matrix(), l3) <= TOL and rel(s.e_field(), e3) <= TOL
        assert s.t == 3
    lr, er = O.leapfrog_n(dim, L, size, links, e, dt, 4)
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.simulate_using_leapfrog_n(dt, 4)
        assert rel(s.link_matrix(), lr) <= TOL and rel(s.e_field(), er) <= TOL


@pytest.mark.parametrize("dim,L", [(2, 5), (3, 4), (4, 3), (4, 4)])
def test_project_to_gauss(oracle_mod, lqgpu_mod, dim, L):
    O, G = oracle_mod, lqgpu_mod
    links, e = random_fields(O, dim, L, 21)
    e_ref, steps_ref = O.project_to_gauss(dim, L, links, e)
    with G.State(dim, L, 1000.0, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        steps = s.project_to_gauss()
        assert steps == steps_ref
        assert rel(s.e_field(), e_ref) <= TOL


@pytest.mark.parametrize("dim,L", [(3, 4), (4, 4)])
def test_project_to_gauss_links_off_the_group(oracle_mod, lqgpu_mod, dim, L):
    """Links that are not exactly unitary (the leap-frog's first-order link update leaves
    |U U^dag - 1| ~ 1e-8 after a trajectory) enter the projection's parallel transports as full
    matrices: U^dag E U then has a trace, and G(x) with it (src/field.rs:1174-1195)."""
    O, G = oracle_mod, lqgpu_mod
    links, e = random_fields(O, dim, L, 23)
    links = links * (1.0 + 1e-6 * np.random.default_rng(5).standard_normal(links.shape))
    e_ref, steps_ref = O.project_to_gauss(dim, L, links, e)
    with G.State(dim, L, 1000.0, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        steps = s.project_to_gauss()
        assert steps == steps_ref
        assert rel(s.e_field(), e_ref) <= TOL


def test_normalize(oracle_mod, lqgpu_mod):
    O, G = oracle_mod, lqgpu_mod
    dim, L = 4, 3
    rng = np.random.default_rng(0)
    links = rng.uniform(-1, 1, size=O.links_shape(dim, L))
    ref = O.normalize(dim, L, links)
    with G.State(dim, L, 1.0, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.normalize_link_matrices()
        assert rel(s.link_matrix(), ref) <= TOL


def test_hmc_trajectories_config1(oracle_mod, lqgpu_mod):
    """HybridMonteCarloDiagnostic on LatticeStateDefault<4>, 8^4, size 1000, beta 1,
    dt 0.01, 10 steps per trajectory, 20 trajectories; momenta N(0, 0.5/beta) and the
    accept uniforms come from the oracle's generator (seed 0) and are injected into both."""
    O, G = oracle_mod, lqgpu_mod
    dim, L, size, beta, dt, nsteps, ntraj = 4, 8, 1000.0, 1.0, 0.01, 10, 20
    rng = O.Rng(0)
    links = O.links_random(dim, L, rng)
    with G.State(dim, L, size, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        for k in range(ntraj):
            e_raw = O.efield_normal(dim, L, rng, 0.5 / beta)
            u = rng.uniform(0.0, 1.0)
            ref = O.hmc_trajectory(dim, L, size, beta, links, e_raw, dt, nsteps, u)
            steps = s.hmc_refresh_upload(e_raw)
            assert steps == ref["gauss_steps"]
            p, h0, h1 = s.hmc_propose(dt, nsteps)
            acc = p >= 1.0 or u < p
            s.hmc_decide(acc)
            assert acc == ref["accepted"]
            assert abs(h0 - ref["h_old"]) <= TOL * abs(ref["h_old"])
            assert abs((h1 - h0) - (ref["h_new"] - ref["h_old"])) <= TOL * abs(ref["h_old"])
            links = ref["links"]
            assert rel(s.link_matrix(), links) <= TOL
            assert abs(s.average_trace_plaquette() - O.average_trace_plaquette(dim, L, links)) <= TOL


@pytest.mark.parametrize("precision", [0, 1])
def test_config1_with_unit_normal_momenta(oracle_mod, lqgpu_mod, precision):
    """The same workload with momenta N(0, 1) in every su(3) component, as the small configuration
    words it (the reference's own draw is N(0, 0.5/beta)): the reference's Gauss projection
    (relaxation 0.12 on a step quadratic in G) diverges at this spread, so the oracle returns
    GaussProjectionError, and so does the library, in FP64 and in the mixed form."""
    O, G = oracle_mod, lqgpu_mod
    dim, L, size, beta, dt, nsteps = 4, 8, 1000.0, 1.0, 0.01, 10
    rng = O.Rng(0)
    links = O.links_random(dim, L, rng)
    e_raw = O.efield_normal(dim, L, rng, 1.0)
    with pytest.raises(O.OracleError) as err:
        O.hmc_trajectory(dim, L, size, beta, links, e_raw, dt, nsteps, 0.5)
    assert err.value.code == O.OR_ERR_GAUSS_PROJECTION
    with G.State(dim, L, size, beta, precision) as s:
        s.set_link_matrix(links)
        with pytest.raises(G.LqError) as gerr:
            s.hmc_refresh_upload(e_raw)
        assert gerr.value.code == G.LQ_ERR_GAUSS_PROJECTION
        # the links are untouched and the state stays usable: a draw at the reference's spread projects
        assert rel(s.link_matrix(), links) <= TOL
        s.hmc_refresh_upload(O.efield_normal(dim, L, rng, 0.5 / beta))


def test_hmc_trajectory_device_rng(lqgpu_mod):
    """The device-RNG trajectory is deterministic in (seed, counter) and keeps links in SU(3)."""
    G = lqgpu_mod
    res = []
    for _ in range(2):
        with G.State(4, 4, 1000.0, 1.0, G.PRECISION_F64) as s:
            s.set_links_random(7)
            r = [s.hmc_trajectory(0.01, 5, 1234, k, 0.5) for k in range(3)]
            res.append((r, s.link_matrix()))
    assert res[0][0] == res[1][0]
    assert np.array_equal(res[0][1], res[1][1])
    assert all(x["gauss_steps"] >= 1 for x in res[0][0])


def test_device_normals_statistics(lqgpu_mod):
    G = lqgpu_mod
    with G.State(4, 8, 1.0, 1.0, G.PRECISION_F64) as s:
        s.set_e_field_normal(42, 0, 0.25)
        e = s.e_field().ravel()
        assert abs(e.mean()) < 5 * 0.25 / np.sqrt(e.size)
        assert abs(e.std() / 0.25 - 1.0) < 0.02
        s.set_e_field_normal(42, 1, 0.25)
        assert not np.array_equal(s.e_field().ravel(), e)


@pytest.mark.parametrize("precision,tol", [(0, 1e-13), (1, 1e-5)])
def test_device_random_links_are_su3(oracle_mod, lqgpu_mod, precision, tol):
    O, G = oracle_mod, lqgpu_mod
    with G.State(3, 4, 1.0, 1.0, precision) as s:
        s.set_links_random(3)
        links = s.link_matrix()
    for m18 in links[::7]:
        m = O.to_complex(m18)
        assert np.abs(m @ m.conj().T - np.eye(3)).max() < tol
        assert abs(np.linalg.det(m) - 1) < 10 * tol


def test_clone_is_independent(oracle_mod, lqgpu_mod):
    O, G = oracle_mod, lqgpu_mod
    links, e = random_fields(O, 3, 4, 9)
    with G.State(3, 4, 5.0, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        c = s.clone()
        s.integrate(G.SYMPLECTIC, 0.1, 2)
        assert np.array_equal(c.link_matrix(), links)
        assert np.array_equal(c.e_field(), e)
        c.close()


def test_errors(oracle_mod, lqgpu_mod):
    G = lqgpu_mod
    with G.State(2, 4, 1.0, 1.0, G.PRECISION_F64) as s:
        with pytest.raises(G.LqError) as ei:
            s.integrate(G.SYMPLECTIC, 0.1, 0)
        assert ei.value.code == G.LQ_ERR_ZERO_INTEGRATION
        with pytest.raises(G.LqError) as ei:
            s.integrate(G.LEAP_LEAP, 0.1, 1)
        assert ei.value.code == G.LQ_ERR_WRONG_STATE_KIND
        with pytest.raises(G.LqError) as ei:
            s.set_link_matrix(np.zeros((3, 18)))
        assert ei.value.code == G.LQ_ERR_INCOMPATIBLE_SIZE
        with pytest.raises(G.LqError) as ei:
            s.set_e_field(np.zeros(5))
        assert ei.value.code == G.LQ_ERR_INCOMPATIBLE_SIZE
        with pytest.raises(G.LqError) as ei:
            s.hmc_decide(True)
        assert ei.value.code == G.LQ_ERR_NO_PENDING
        with pytest.raises(G.LqError) as ei:
            s.hmc_propose(0.1, 0)
        assert ei.value.code == G.LQ_ERR_ZERO_INTEGRATION
        s.set_beta(0.0)
        with pytest.raises(G.LqError) as ei:
            s.hmc_refresh(1, 0)
        assert ei.value.code == G.LQ_ERR_INVALID_NORMAL
        s.set_beta(1.0)
        e = np.zeros((16, 2, 8))
        e[3, 1, 2] = np.nan
        with pytest.raises(G.LqError) as ei:
            s.hmc_refresh_upload(e)
        assert ei.value.code == G.LQ_ERR_GAUSS_PROJECTION
        s.set_links_random(1)
        s.set_e_field_normal(1, 0, 0.5)
        with pytest.raises(G.LqError) as ei:
            s.project_to_gauss(max_steps=3)
        assert ei.value.code == G.LQ_ERR_NOT_CONVERGED
        # the context is still usable after every error
        assert s.hamiltonian_links() >= 0.0
