"""FP64 parity with the CPU oracle on the large lattices whose index paths the 32^4 workload runs.

The small cases of test_parity_gpu.py (L <= 8) never reach the code paths that only appear at
large L: the site decode by multiplication (divisor_magic) at L = 16 and 32, rows of exactly one
32-site tile (L = 32: the x0 neighbour of lane 31 is lane 0 of the same tile), x1 neighbours
one whole tile away, and the directions-fastest block order over many site blocks.  These tests
run those paths against the oracle with the same injected links and momenta.

Tolerances as in test_parity_gpu.py: 1e-12 relative to max(1, |value|) per link and momentum
coefficient, 1e-12 * |H| for Hamiltonians and Delta H.  The mixed form is compared with the
oracle at 32^4 too, with the FP32 tolerance written below.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12
# mixed form after two symplectic steps at size 7 (links move ~1e-2 per step): every product in
# FP32 (epsilon 6e-8) on O(1) entries, the stored state compensated
TOL_MIXED = 2e-6


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(1.0, float(np.abs(b).max())))


@pytest.fixture(scope="module")
def threads(oracle_mod):
    import os

    oracle_mod.set_threads(os.cpu_count() or 1)
    return oracle_mod.get_threads()


def _trajectory_case(O, G, dim, L, seed, size, beta, dt, nsteps):
    rng = O.Rng(seed)
    links = O.links_random(dim, L, rng)
    e_raw = O.efield_normal(dim, L, rng, 0.5 / beta)
    u = rng.uniform(0.0, 1.0)
    ref = O.hmc_trajectory(dim, L, size, beta, links, e_raw, dt, nsteps, u)
    with G.State(dim, L, size, beta, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        steps = s.hmc_refresh_upload(e_raw)
        assert steps == ref["gauss_steps"]
        p, h0, h1 = s.hmc_propose(dt, nsteps)
        acc = p >= 1.0 or u < p
        assert acc == ref["accepted"]
        assert abs(h0 - ref["h_old"]) <= TOL * abs(ref["h_old"])
        assert abs(h1 - ref["h_new"]) <= TOL * abs(ref["h_old"])
        assert abs((h1 - h0) - (ref["h_new"] - ref["h_old"])) <= TOL * abs(ref["h_old"])
        s.hmc_decide(acc)
        assert rel(s.link_matrix(), ref["links"]) <= TOL
        p_ref = O.average_trace_plaquette(dim, L, ref["links"])
        assert abs(s.average_trace_plaquette() - p_ref) <= TOL
    return ref


def test_trajectory_16x4(oracle_mod, lqgpu_mod, threads):
    """one full HMC trajectory at D = 4, 16^4 (projection, 5 MD steps, both Hamiltonians, accept)"""
    ref = _trajectory_case(oracle_mod, lqgpu_mod, 4, 16, 16, 1000.0, 2.0, 0.005, 5)
    assert ref["gauss_steps"] >= 5


def test_trajectory_32x3(oracle_mod, lqgpu_mod, threads):
    """one full HMC trajectory at D = 3, 32^3: rows of one tile, x1 neighbours one tile away"""
    _trajectory_case(oracle_mod, lqgpu_mod, 3, 32, 32, 1000.0, 2.0, 0.005, 5)


@pytest.fixture(scope="module")
def fields_32x4(oracle_mod, threads):
    O = oracle_mod
    dim, L, size, dt = 4, 32, 7.0, 0.02
    rng = O.Rng(324)
    links = O.links_random(dim, L, rng)
    e = O.efield_normal(dim, L, rng, 0.25)
    lr, er = O.integrate(dim, L, size, links, e, O.SYMPLECTIC, dt, 2)
    return dict(dim=dim, L=L, size=size, dt=dt, links=links, e=e, lr=lr, er=er)


def test_integrate_symplectic_32x4(oracle_mod, lqgpu_mod, fields_32x4):
    """two symplectic steps at D = 4, 32^4 from injected links and momenta (no projection, so the
    oracle's time stays bounded): links, momenta, both Hamiltonians and the plaquette"""
    O, G, f = oracle_mod, lqgpu_mod, fields_32x4
    dim, L, beta = f["dim"], f["L"], 2.0
    with G.State(dim, L, f["size"], beta, G.PRECISION_F64) as s:
        s.set_link_matrix(f["links"])
        s.set_e_field(f["e"])
        s.integrate(G.SYMPLECTIC, f["dt"], 2)
        assert rel(s.link_matrix(), f["lr"]) <= TOL
        assert rel(s.e_field(), f["er"]) <= TOL
        hu_ref = O.hamiltonian_links(dim, L, beta, f["lr"])
        he_ref = O.hamiltonian_efield(dim, L, beta, f["er"])
        assert abs(s.hamiltonian_links() - hu_ref) <= TOL * abs(hu_ref)
        assert abs(s.hamiltonian_efield() - he_ref) <= TOL * abs(he_ref)
        assert abs(s.average_trace_plaquette() - O.average_trace_plaquette(dim, L, f["lr"])) <= TOL


@pytest.mark.parametrize("precision", ["mixed", "f32"])
def test_integrate_symplectic_32x4_fp32_forms(oracle_mod, lqgpu_mod, fields_32x4, precision):
    """the FP32-arithmetic forms on the same 32^4 inputs, against the oracle"""
    G, f = lqgpu_mod, fields_32x4
    prec = {"mixed": G.PRECISION_MIXED, "f32": G.PRECISION_F32}[precision]
    with G.State(f["dim"], f["L"], f["size"], 2.0, prec) as s:
        s.set_link_matrix(f["links"])
        s.set_e_field(f["e"])
        s.integrate(G.SYMPLECTIC, f["dt"], 2)
        assert rel(s.link_matrix(), f["lr"]) <= TOL_MIXED
        assert rel(s.e_field(), f["er"]) <= TOL_MIXED
