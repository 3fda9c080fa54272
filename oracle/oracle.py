"""ctypes binding of the C++ oracle (``lq_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: used by the tests, the smoke check and bench.py's CPU
baseline.  Arrays use the reference's serde layouts:

* links  ``float64[V*D, 18]``: per link a column-major 3x3 complex matrix, (re, im)
* efield ``float64[V, D, 8]``: su(3) coefficients per site and direction
"""
import ctypes
import os

import numpy as np

from . import build_oracle

OR_OK = 0
OR_ERR_NON_POSITIVE_SIZE = 1
OR_ERR_DIM_TOO_SMALL = 2
OR_ERR_ZERO_DIMENSION = 3
OR_ERR_UNSUPPORTED_D = 4
OR_ERR_INVALID_NORMAL = 5
OR_ERR_GAUSS_PROJECTION = 7
OR_ERR_ZERO_INTEGRATION = 8
OR_ERR_INVALID_ARGUMENT = 9
OR_ERR_NOT_CONVERGED = 10

SYNC_SYNC, SYNC_LEAP, LEAP_LEAP, LEAP_SYNC, SYMPLECTIC, SYMPLECTIC_EXP, SYMPLECTIC_EXP_NORMALIZE = range(7)

_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


class OracleError(RuntimeError):
    def __init__(self, code, what):
        super().__init__("%s failed with oracle status %d" % (what, code))
        self.code = code


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.LIB
        if not os.path.exists(path):
            path = build_oracle.build()
        L = ctypes.CDLL(path)
        vp, i32, u64, f64, lng = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_double, ctypes.c_long
        ip = ctypes.POINTER(ctypes.c_int)
        sig = {
            "or_rng_new": (vp, [u64]),
            "or_rng_free": (None, [vp]),
            "or_rng_next_u64": (u64, [vp]),
            "or_rng_uniform": (f64, [vp, f64, f64]),
            "or_rng_standard_normal": (f64, [vp]),
            "or_lattice_new": (i32, [i32, f64, lng]),
            "or_generators": (None, [_dp]),
            "or_su3_to_matrix": (None, [_dp, _dp]),
            "or_su3_exp_i": (None, [_dp, _dp]),
            "or_su3_exp_r": (None, [_dp, _dp]),
            "or_orthonormalize": (None, [_dp, _dp]),
            "or_random_su3": (None, [vp, _dp]),
            "or_matmul": (None, [_dp, _dp, _dp]),
            "or_determinant": (None, [_dp, _dp]),
            "or_links_random": (i32, [i32, i32, vp, _dp]),
            "or_links_cold": (i32, [i32, i32, _dp]),
            "or_efield_normal": (i32, [i32, i32, vp, f64, _dp]),
            "or_hamiltonian_links": (i32, [i32, i32, f64, _dp, _dp]),
            "or_hamiltonian_efield": (i32, [i32, i32, f64, _dp, _dp]),
            "or_average_trace_plaquette": (i32, [i32, i32, _dp, _dp, _dp]),
            "or_gauss": (i32, [i32, i32, _dp, _dp, lng, _dp]),
            "or_clover": (i32, [i32, i32, _dp, lng, i32, i32, i32, i32, _dp]),
            "or_metropolis_sweep": (i32, [i32, i32, ctypes.c_double, _dp, i32, ctypes.c_double, u64, u64, _dp,
                                          ctypes.POINTER(ctypes.c_long), _dp]),
            "or_heat_bath_sweep": (i32, [i32, i32, ctypes.c_double, _dp, u64, u64, _dp]),
            "or_overrelaxation_sweep": (i32, [i32, i32, _dp, i32, _dp]),
            "or_overrelax_link": (i32, [_dp, _dp, i32, _dp]),
            "or_f_mu_nu": (i32, [i32, i32, ctypes.c_double, _dp, lng, i32, i32, _dp]),
            "or_magnetic_field": (i32, [i32, i32, ctypes.c_double, _dp, lng, i32, _dp]),
            "or_gauss_sum_div": (i32, [i32, i32, _dp, _dp, _dp]),
            "or_project_to_gauss": (i32, [i32, i32, _dp, _dp, _dp, i32, ip]),
            "or_normalize": (i32, [i32, i32, _dp]),
            "or_derivative_e": (i32, [i32, i32, f64, _dp, _dp]),
            "or_derivative_u": (i32, [i32, i32, f64, _dp, _dp, _dp]),
            "or_integrate": (i32, [i32, i32, f64, _dp, _dp, i32, f64, i32, _dp, _dp]),
            "or_leapfrog_n": (i32, [i32, i32, f64, _dp, _dp, f64, i32, _dp, _dp]),
            "or_hmc_trajectory": (i32, [i32, i32, f64, f64, _dp, _dp, f64, i32, f64, i32, _dp, _dp,
                                        ip, _dp, _dp, _dp, ip]),
            "or_set_threads": (None, [i32]),
            "or_get_threads": (i32, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _check(code, what):
    if code != OR_OK:
        raise OracleError(code, what)


def n_sites(dim, L):
    return L ** dim


def links_shape(dim, L):
    return (n_sites(dim, L) * dim, 18)


def efield_shape(dim, L):
    return (n_sites(dim, L), dim, 8)


class Rng:
    """Xoshiro256++ seeded through SplitMix64."""

    def __init__(self, seed):
        self._h = lib().or_rng_new(ctypes.c_uint64(seed & (2 ** 64 - 1)))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.or_rng_free(self._h)
            self._h = None

    def next_u64(self):
        return lib().or_rng_next_u64(self._h)

    def uniform(self, low=0.0, high=1.0):
        return lib().or_rng_uniform(self._h, low, high)

    def standard_normal(self):
        return lib().or_rng_standard_normal(self._h)


def lattice_new(dim, size, L):
    return lib().or_lattice_new(dim, size, L)


def generators():
    out = np.zeros((8, 18))
    lib().or_generators(_p(out))
    return out


def _adj_to_mat(fn, adj):
    adj = np.ascontiguousarray(adj, dtype=np.float64)
    out = np.zeros(18)
    fn(_p(adj), _p(out))
    return out


def su3_to_matrix(adj):
    return _adj_to_mat(lib().or_su3_to_matrix, adj)


def su3_exp_i(adj):
    return _adj_to_mat(lib().or_su3_exp_i, adj)


def su3_exp_r(adj):
    return _adj_to_mat(lib().or_su3_exp_r, adj)


def orthonormalize(m18):
    return _adj_to_mat(lib().or_orthonormalize, m18)


def random_su3(rng):
    out = np.zeros(18)
    lib().or_random_su3(rng._h, _p(out))
    return out


def matmul(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros(18)
    lib().or_matmul(_p(a), _p(b), _p(out))
    return out


def determinant(m):
    m = np.ascontiguousarray(m, dtype=np.float64)
    out = np.zeros(2)
    lib().or_determinant(_p(m), _p(out))
    return complex(out[0], out[1])


def links_random(dim, L, rng):
    out = np.zeros(links_shape(dim, L))
    _check(lib().or_links_random(dim, L, rng._h, _p(out)), "links_random")
    return out


def links_cold(dim, L):
    out = np.zeros(links_shape(dim, L))
    _check(lib().or_links_cold(dim, L, _p(out)), "links_cold")
    return out


def efield_normal(dim, L, rng, std_dev):
    out = np.zeros(efield_shape(dim, L))
    _check(lib().or_efield_normal(dim, L, rng._h, std_dev, _p(out)), "efield_normal")
    return out


def hamiltonian_links(dim, L, beta, links):
    out = np.zeros(1)
    _check(lib().or_hamiltonian_links(dim, L, beta, _p(links), _p(out)), "hamiltonian_links")
    return float(out[0])


def hamiltonian_efield(dim, L, beta, efield):
    out = np.zeros(1)
    _check(lib().or_hamiltonian_efield(dim, L, beta, _p(efield), _p(out)), "hamiltonian_efield")
    return float(out[0])


def average_trace_plaquette(dim, L, links):
    re, im = np.zeros(1), np.zeros(1)
    _check(lib().or_average_trace_plaquette(dim, L, _p(links), _p(re), _p(im)), "average_trace_plaquette")
    return complex(re[0], im[0])


def gauss(dim, L, links, efield, site):
    out = np.zeros(18)
    _check(lib().or_gauss(dim, L, _p(links), _p(efield), site, _p(out)), "gauss")
    return out


def metropolis_sweep(dim, L, beta, links, n_update, spread, seed, sweep):
    """checkerboard MetropolisHastingsSweep with the per-link Philox stream; (links, accepted, sum p)"""
    out = np.zeros_like(links)
    acc = ctypes.c_long(0)
    ps = np.zeros(1)
    _check(lib().or_metropolis_sweep(dim, L, beta, _p(np.ascontiguousarray(links)), n_update, spread, seed, sweep,
                                     _p(out), ctypes.byref(acc), _p(ps)), "metropolis_sweep")
    return out, acc.value, float(ps[0])


def heat_bath_sweep(dim, L, beta, links, seed, sweep):
    """checkerboard HeatBathSweep with the per-link Philox stream"""
    out = np.zeros_like(links)
    _check(lib().or_heat_bath_sweep(dim, L, beta, _p(np.ascontiguousarray(links)), seed, sweep, _p(out)),
           "heat_bath_sweep")
    return out


def overrelaxation_sweep(dim, L, links, method):
    """checkerboard OverrelaxationSweepRotation (method 0) / OverrelaxationSweepReverse (1)"""
    out = np.zeros_like(links)
    _check(lib().or_overrelaxation_sweep(dim, L, _p(np.ascontiguousarray(links)), method, _p(out)),
           "overrelaxation_sweep")
    return out


def overrelax_link(link18, staple18, method):
    """one link's overrelaxation update from its link and staple matrices (18 doubles each)"""
    out = np.zeros(18)
    _check(lib().or_overrelax_link(_p(np.ascontiguousarray(link18, dtype=np.float64)),
                                   _p(np.ascontiguousarray(staple18, dtype=np.float64)), method, _p(out)),
           "overrelax_link")
    return out


def clover(dim, L, links, site, i, j, i_positive=True, j_positive=True):
    """LinkMatrix::clover (src/field.rs:806-820) at one point, 18 doubles"""
    out = np.zeros(18)
    _check(lib().or_clover(dim, L, _p(links), site, i, int(i_positive), j, int(j_positive), _p(out)), "clover")
    return out


def f_mu_nu(dim, L, size, links, site, i, j):
    """LinkMatrix::f_mu_nu (src/field.rs:822-835), positive directions"""
    out = np.zeros(18)
    _check(lib().or_f_mu_nu(dim, L, size, _p(links), site, i, j, _p(out)), "f_mu_nu")
    return out


def magnetic_field(dim, L, size, links, site, k):
    """LinkMatrix::magnetic_field (src/field.rs:849-871) along positive direction k"""
    out = np.zeros(18)
    _check(lib().or_magnetic_field(dim, L, size, _p(links), site, k, _p(out)), "magnetic_field")
    return out


def gauss_sum_div(dim, L, links, efield):
    out = np.zeros(1)
    _check(lib().or_gauss_sum_div(dim, L, _p(links), _p(efield), _p(out)), "gauss_sum_div")
    return float(out[0])


def project_to_gauss(dim, L, links, efield, max_steps=100000):
    out = np.zeros(efield_shape(dim, L))
    steps = ctypes.c_int(0)
    _check(lib().or_project_to_gauss(dim, L, _p(links), _p(efield), _p(out), max_steps, ctypes.byref(steps)),
           "project_to_gauss")
    return out, steps.value


def normalize(dim, L, links):
    out = np.array(links, dtype=np.float64, copy=True)
    _check(lib().or_normalize(dim, L, _p(out)), "normalize")
    return out


def derivative_e(dim, L, size, links):
    out = np.zeros(efield_shape(dim, L))
    _check(lib().or_derivative_e(dim, L, size, _p(links), _p(out)), "derivative_e")
    return out


def derivative_u(dim, L, size, links, efield):
    out = np.zeros(links_shape(dim, L))
    _check(lib().or_derivative_u(dim, L, size, _p(links), _p(efield), _p(out)), "derivative_u")
    return out


def integrate(dim, L, size, links, efield, mode, dt, n):
    lo = np.zeros(links_shape(dim, L))
    eo = np.zeros(efield_shape(dim, L))
    _check(lib().or_integrate(dim, L, size, _p(links), _p(efield), mode, dt, n, _p(lo), _p(eo)), "integrate")
    return lo, eo


def leapfrog_n(dim, L, size, links, efield, dt, n):
    lo = np.zeros(links_shape(dim, L))
    eo = np.zeros(efield_shape(dim, L))
    _check(lib().or_leapfrog_n(dim, L, size, _p(links), _p(efield), dt, n, _p(lo), _p(eo)), "leapfrog_n")
    return lo, eo


def hmc_trajectory(dim, L, size, beta, links, efield_raw, dt, n_steps, uniform, max_gauss_steps=100000):
    """One HybridMonteCarloDiagnostic step with injected momenta and uniform draw."""
    lo = np.zeros(links_shape(dim, L))
    eo = np.zeros(efield_shape(dim, L))
    acc = ctypes.c_int(0)
    gs = ctypes.c_int(0)
    prob, h0, h1 = np.zeros(1), np.zeros(1), np.zeros(1)
    _check(lib().or_hmc_trajectory(dim, L, size, beta, _p(links), _p(efield_raw), dt, n_steps, uniform,
                                   max_gauss_steps, _p(lo), _p(eo), ctypes.byref(acc), _p(prob), _p(h0), _p(h1),
                                   ctypes.byref(gs)), "hmc_trajectory")
    return dict(links=lo, efield=eo, accepted=bool(acc.value), prob=float(prob[0]), h_old=float(h0[0]),
                h_new=float(h1[0]), gauss_steps=gs.value)


def set_threads(n):
    lib().or_set_threads(n)


def get_threads():
    return lib().or_get_threads()


# ---- helpers on the serde layout ----
def to_complex(m18):
    """18 doubles (column-major, re/im) -> 3x3 complex ndarray [row, col]."""
    m = np.asarray(m18, dtype=np.float64).reshape(3, 3, 2)  # [col, row, re/im]
    return (m[..., 0] + 1j * m[..., 1]).T


def from_complex(c):
    c = np.asarray(c, dtype=np.complex128).T  # [col, row]
    out = np.zeros((3, 3, 2))
    out[..., 0] = c.real
    out[..., 1] = c.imag
    return out.reshape(18)
