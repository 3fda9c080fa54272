"""Clover observables on the device (lq_field_strength, lq_magnetic_field) against the oracle's
restatement of LinkMatrix::clover / f_mu_nu / magnetic_field (src/field.rs:806-871) at every
site, FP64 (1e-12 of the largest entry), and the reference's own known answers
(src/field.rs:1579-1711) through the device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,L", [(2, 4), (3, 3), (4, 3)])
def test_fields_match_oracle(oracle_mod, lqgpu_mod, dim, L):
    O, G = oracle_mod, lqgpu_mod
    size = 2.5
    links = O.links_random(dim, L, O.Rng(13))
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        f = s.field_strength()
        b = s.magnetic_field()
    planes = [(i, j) for i in range(dim) for j in range(i + 1, dim)]
    fr = np.array([[O.f_mu_nu(dim, L, size, links, x, i, j) for (i, j) in planes] for x in range(L ** dim)])
    br = np.array([[O.magnetic_field(dim, L, size, links, x, k) for k in range(dim)] for x in range(L ** dim)])
    assert np.abs(f - fr).max() <= 1e-12 * max(1.0, np.abs(fr).max())
    assert np.abs(b - br).max() <= 1e-12 * max(1.0, np.abs(br).max())
    if dim == 2:
        assert not b.any()


def test_known_answers_through_the_device(oracle_mod, lqgpu_mod):
    O, G = oracle_mod, lqgpu_mod
    dim, L, size = 3, 4, 1.0
    I3 = np.eye(3)
    links = O.links_cold(dim, L)
    links[1 * dim + 1] = O.from_complex(1j * I3)  # site [1, 0, 0], direction y
    with G.State(dim, L, size, 1.0, G.PRECISION_F64) as s:
        s.set_link_matrix(links)
        f = s.field_strength()
        b = s.magnetic_field()
    assert np.abs(O.to_complex(f[0, 0]) - 0.25j * I3).max() <= 1e-15  # F_xy at the origin
    assert np.abs(O.to_complex(b[0, 2]) - 0.25 * I3).max() <= 1e-15
    assert np.abs(b[0, :2]).max() <= 1e-15


@pytest.mark.parametrize("precision", [1, 2])
def test_fp32_forms(oracle_mod, lqgpu_mod, precision):
    O, G = oracle_mod, lqgpu_mod
    links = O.links_random(4, 4, O.Rng(3))
    out = []
    for p in (G.PRECISION_F64, precision):
        with G.State(4, 4, 1.0, 1.0, p) as s:
            s.set_link_matrix(links)
            out.append((s.field_strength(), s.magnetic_field()))
    assert np.abs(out[1][0] - out[0][0]).max() <= 1e-5
    assert np.abs(out[1][1] - out[0][1]).max() <= 1e-5
