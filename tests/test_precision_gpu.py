"""The FP32-arithmetic forms against the FP64 form, from identical links, momenta and
accept uniforms.

Tolerances written here (8^4, size 1000, beta 2, dt 0.005, 20 steps, 4 trajectories):
* mixed (compensated FP32 pairs): |Delta H - Delta H_f64| <= 1e-6, |<P>/3 - <P>/3_f64| <= 1e-7
  (the spec bar at 32^4 is 1e-4 and 1e-6);
* f32 (plain FP32 storage): |Delta H error| <= 1e-2 and plaquette <= 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(G, precision, links, moms, us, dim, L, size, beta, dt, n):
    out = []
    with G.State(dim, L, size, beta, precision) as s:
        s.set_link_matrix(links)
        for e_raw, u in zip(moms, us):
            steps = s.hmc_refresh_upload(e_raw)
            p, h0, h1 = s.hmc_propose(dt, n)
            acc = p >= 1.0 or u < p
            s.hmc_decide(acc)
            out.append(dict(dh=h1 - h0, h0=h0, acc=acc, steps=steps, plaq=s.average_trace_plaquette().real / 3.0))
        final = s.link_matrix()
    return out, final


@pytest.mark.parametrize("precision,dh_tol,plaq_tol", [(1, 1e-6, 1e-7), (2, 1e-2, 1e-5)])
def test_precision_against_fp64(oracle_mod, lqgpu_mod, precision, dh_tol, plaq_tol):
    O, G = oracle_mod, lqgpu_mod
    dim, L, size, beta, dt, n = 4, 8, 1000.0, 2.0, 0.005, 20
    rng = O.Rng(1)
    links = O.links_random(dim, L, rng)
    moms = [O.efield_normal(dim, L, rng, 0.5 / beta) for _ in range(4)]
    us = [rng.uniform(0, 1) for _ in range(4)]
    ref, _ = run(G, G.PRECISION_F64, links, moms, us, dim, L, size, beta, dt, n)
    got, final = run(G, precision, links, moms, us, dim, L, size, beta, dt, n)
    for r, g in zip(ref, got):
        assert abs(g["dh"] - r["dh"]) <= dh_tol, (g["dh"], r["dh"])
        assert abs(g["plaq"] - r["plaq"]) <= plaq_tol
        assert abs(g["h0"] - r["h0"]) <= 1e-6 * abs(r["h0"])
        assert g["acc"] == r["acc"]


def test_mixed_roundtrip_keeps_48_bits(oracle_mod, lqgpu_mod):
    O, G = oracle_mod, lqgpu_mod
    rng = O.Rng(2)
    links = O.links_random(3, 4, rng)
    e = O.efield_normal(3, 4, rng, 0.7)
    with G.State(3, 4, 1.0, 1.0, G.PRECISION_MIXED) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        # a double split into two FP32 keeps 48 bits: relative error <= 2^-48
        assert np.abs(s.link_matrix() - links).max() <= 4e-15 * np.abs(links).max()
        assert np.abs(s.e_field() - e).max() <= 4e-15 * np.abs(e).max()


@pytest.mark.parametrize("precision", [1, 2])
def test_fp32_forms_track_the_fp64_integrator(oracle_mod, lqgpu_mod, precision):
    """One symplectic_n integration (size 3, dt 0.02: large increments) from identical fields.
    The increments carry FP32 relative error in both forms; mixed adds no rounding of the
    stored state.  Bounds: mixed 1e-6, f32 1e-5 (absolute, entries O(1))."""
    O, G = oracle_mod, lqgpu_mod
    dim, L, size, dt, n = 4, 4, 3.0, 0.02, 10
    rng = O.Rng(3)
    links = O.links_random(dim, L, rng)
    e = O.efield_normal(dim, L, rng, 0.5)
    lr, er = O.integrate(dim, L, size, links, e, O.SYMPLECTIC, dt, n)
    with G.State(dim, L, size, 1.0, precision) as s:
        s.set_link_matrix(links)
        s.set_e_field(e)
        s.integrate(G.SYMPLECTIC, dt, n)
        tol = 1e-6 if precision == G.PRECISION_MIXED else 1e-5
        du, de = np.abs(s.link_matrix() - lr).max(), np.abs(s.e_field() - er).max()
        print("precision", precision, "link error", du, "E error", de)
        assert du <= tol and de <= tol


def test_mixed_reprojection_in_fp64(oracle_mod, lqgpu_mod):
    O, G = oracle_mod, lqgpu_mod
    rng = np.random.default_rng(4)
    links = rng.uniform(-1, 1, size=O.links_shape(3, 3))
    ref = O.normalize(3, 3, links)
    with G.State(3, 3, 1.0, 1.0, G.PRECISION_MIXED) as s:
        s.set_link_matrix(links)
        s.normalize_link_matrices()
        assert np.abs(s.link_matrix() - ref).max() <= 1e-13
