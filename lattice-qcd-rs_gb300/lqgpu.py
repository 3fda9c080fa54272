"""ctypes binding of liblqgpu.so (the C ABI declared in include/lqgpu.h).

The binding loads the in-tree CUDA library and nothing else: there is no CPU fallback.
If the library is missing, or no CUDA device is visible when a state is created, the
calls raise :class:`LqError`.

Arrays use the reference crate's serde layouts (lattice-qcd-rs v0.2.1):

* links  ``float64[V*D, 18]`` -- per link (index site*D + mu) a column-major 3x3 complex
  matrix stored as (re, im) pairs (nalgebra ``Matrix3<Complex<f64>>``);
* efield ``float64[V, D, 8]`` -- su(3) coefficients e^a of E = e^a T^a.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "liblqgpu.so")

LQ_OK = 0
STATUS = {
    0: "LQ_OK", 1: "LQ_ERR_NON_POSITIVE_SIZE", 2: "LQ_ERR_DIM_TOO_SMALL", 3: "LQ_ERR_ZERO_DIMENSION",
    4: "LQ_ERR_UNSUPPORTED_DIM", 5: "LQ_ERR_INVALID_NORMAL", 6: "LQ_ERR_INCOMPATIBLE_SIZE",
    7: "LQ_ERR_GAUSS_PROJECTION", 8: "LQ_ERR_ZERO_INTEGRATION", 9: "LQ_ERR_INVALID_ARGUMENT",
    10: "LQ_ERR_NOT_CONVERGED", 11: "LQ_ERR_WRONG_STATE_KIND", 12: "LQ_ERR_NO_PENDING", 20: "LQ_ERR_CUDA",
    21: "LQ_ERR_OUT_OF_MEMORY", 22: "LQ_ERR_NO_DEVICE",
}
globals().update({v: k for k, v in STATUS.items()})

PRECISION_F64 = 0
PRECISION_MIXED = 1
PRECISION_F32 = 2
SYNC_SYNC, SYNC_LEAP, LEAP_LEAP, LEAP_SYNC, SYMPLECTIC, SYMPLECTIC_EXP, SYMPLECTIC_EXP_REUNITARIZE = range(7)
LINK_UPDATE_EULER, LINK_UPDATE_EXP, LINK_UPDATE_EXP_REUNITARIZE = range(3)
OVERRELAX_ROTATION, OVERRELAX_REVERSE = range(2)
BATCH_USE_GRAPH, BATCH_MEASURE_PLAQUETTE = 1, 2
BATCH_KERNEL_CLASSES = ("md", "sweep", "gauss", "plaquette_delta", "sumsq_delta", "normal", "plaquette")

# every symbol the header declares, with (restype, argtypes)
_vp, _i32, _u64, _f64, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_double, ctypes.c_size_t
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_llp = ctypes.POINTER(ctypes.c_longlong)
_szp = ctypes.POINTER(ctypes.c_size_t)
SIGNATURES = {
    "lq_state_create": (_i32, [_i32, _i32, _f64, _f64, _i32, ctypes.POINTER(_vp)]),
    "lq_state_destroy": (_i32, [_vp]),
    "lq_state_clone": (_i32, [_vp, ctypes.POINTER(_vp)]),
    "lq_state_checkpoint_bytes": (_i32, [_vp, _szp]),
    "lq_state_save": (_i32, [_vp, _vp, _sz]),
    "lq_state_load": (_i32, [_vp, _sz, ctypes.POINTER(_vp)]),
    "lq_state_set_stream": (_i32, [_vp, _vp]),
    "lq_state_set_projection_graph": (_i32, [_vp, _i32]),
    "lq_state_info": (_i32, [_vp, _ip, _ip, _dp, _dp, _ip, _llp, _llp, _ip]),
    "lq_state_set_beta": (_i32, [_vp, _f64]),
    "lq_state_set_link_update": (_i32, [_vp, _i32]),
    "lq_state_device_bytes": (_i32, [_vp, _szp]),
    "lq_links_upload": (_i32, [_vp, _dp, _sz]),
    "lq_links_download": (_i32, [_vp, _dp, _sz]),
    "lq_links_set_cold": (_i32, [_vp]),
    "lq_links_random": (_i32, [_vp, _u64]),
    "lq_efield_upload": (_i32, [_vp, _dp, _sz]),
    "lq_efield_download": (_i32, [_vp, _dp, _sz]),
    "lq_efield_set_cold": (_i32, [_vp]),
    "lq_efield_random_normal": (_i32, [_vp, _u64, _u64, _f64]),
    "lq_hamiltonian_links": (_i32, [_vp, _dp]),
    "lq_hamiltonian_efield": (_i32, [_vp, _dp]),
    "lq_hamiltonian_total": (_i32, [_vp, _dp]),
    "lq_average_trace_plaquette": (_i32, [_vp, _dp, _dp]),
    "lq_gauss_sum_div": (_i32, [_vp, _dp]),
    "lq_gauss_download": (_i32, [_vp, _dp, _sz]),
    "lq_project_gauss": (_i32, [_vp, _i32, _ip]),
    "lq_normalize_link_matrices": (_i32, [_vp]),
    "lq_integrate": (_i32, [_vp, _i32, _f64, _i32]),
    "lq_leapfrog_n": (_i32, [_vp, _f64, _i32]),
    "lq_hmc_refresh": (_i32, [_vp, _u64, _u64, _i32, _ip]),
    "lq_hmc_refresh_upload": (_i32, [_vp, _dp, _sz, _i32, _ip]),
    "lq_efield_prefetch": (_i32, [_vp, _dp, _sz]),
    "lq_hmc_refresh_prefetched": (_i32, [_vp, _i32, _ip]),
    "lq_hmc_propose": (_i32, [_vp, _f64, _i32, _dp, _dp, _dp]),
    "lq_hmc_decide": (_i32, [_vp, _i32]),
    "lq_hmc_trajectory": (_i32, [_vp, _f64, _i32, _u64, _u64, _f64, _i32, _ip, _dp, _dp, _ip]),
    "lq_plaquette_sums_noalloc": (_i32, [_i32, _i32, _vp, _vp, _vp]),
    "lq_wilson_action": (_i32, [_vp, _dp]),
    "lq_wilson_action_backward": (_i32, [_vp, _dp, _sz]),
    "lq_link_rotate": (_i32, [_vp, ctypes.c_longlong, _i32, _f64]),
    "lq_metropolis_sweep": (_i32, [_vp, _i32, _f64, _u64, _u64, _llp, _dp]),
    "lq_heat_bath_sweep": (_i32, [_vp, _u64, _u64]),
    "lq_overrelaxation_sweep": (_i32, [_vp, _i32]),
    "lq_field_strength": (_i32, [_vp, _dp, _sz]),
    "lq_magnetic_field": (_i32, [_vp, _dp, _sz]),
    "lq_leapfrog_adjoint": (_i32, [_vp, _f64, _i32, _i32, _dp, _dp, _dp, _sz, _dp, _sz, _szp]),
    "lq_profile_enable": (_i32, [_vp, _i32]),
    "lq_profile_classes": (_i32, [_vp, ctypes.c_uint]),
    "lq_bounds_check": (_i32, [_ip, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong), _i32]),
    "lq_profile_read": (_i32, [_vp, _i32, _llp, _dp, _i32]),
    "lq_fma_peak": (_i32, [_i32, _dp]),
    "lq_batch_create": (_i32, [_i32, _i32, _ip, _dp, _dp, _i32, ctypes.POINTER(_vp)]),
    "lq_batch_destroy": (_i32, [_vp]),
    "lq_batch_set_stream": (_i32, [_vp, _vp]),
    "lq_batch_info": (_i32, [_vp, _ip, _ip, _llp, _szp]),
    "lq_batch_set_link_update": (_i32, [_vp, _i32]),
    "lq_batch_set_seed": (_i32, [_vp, _u64, _u64]),
    "lq_batch_links_random": (_i32, [_vp, _u64]),
    "lq_batch_links_upload": (_i32, [_vp, _i32, _dp, _sz]),
    "lq_batch_links_download": (_i32, [_vp, _i32, _dp, _sz]),
    "lq_batch_normalize_link_matrices": (_i32, [_vp]),
    "lq_batch_average_trace_plaquette": (_i32, [_vp, _dp, _dp]),
    "lq_batch_autotune": (_i32, [_vp, _f64, _i32]),
    "lq_batch_tuning": (_i32, [_vp, _i32, _ip, _ip, _dp]),
    "lq_batch_hmc_run": (_i32, [_vp, _f64, _i32, _i32, _i32, _i32]),
    "lq_batch_hmc_results": (_i32, [_vp, _i32, _i32, _dp, _dp, _dp, _ip, _ip, _ip, _dp]),
    "lq_batch_graph_launches": (_i32, [_vp, _llp]),
    "lq_batch_profile_enable": (_i32, [_vp, _i32]),
    "lq_batch_profile_read": (_i32, [_vp, _llp, _dp, _i32]),
    "lq_status_string": (ctypes.c_char_p, [_i32]),
    "lq_last_error_string": (ctypes.c_char_p, []),
    "lq_version": (_i32, []),
}

_lib = None


class LqError(RuntimeError):
    def __init__(self, code, what, detail=""):
        name = STATUS.get(code, str(code))
        msg = "%s failed: %s" % (what, name)
        if detail:
            msg += " (%s)" % detail
        super().__init__(msg)
        self.code = code


def load(path=None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise LqError(-1, "load", "CUDA library %s is missing; run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(code, what):
    if code != LQ_OK:
        detail = ""
        if code in (20, 21, 22):
            detail = load().lq_last_error_string().decode()
        raise LqError(code, what, detail)


def _p(a):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_dp)


class State:
    """A device-resident LatticeStateEFSyncDefault<LatticeStateDefault<D>, D>."""

    def __init__(self, dim, L, size=1000.0, beta=1.0, precision=PRECISION_F64, _handle=None):
        lib = load()
        if _handle is None:
            h = _vp()
            _check(lib.lq_state_create(dim, L, size, beta, precision, ctypes.byref(h)), "lq_state_create")
            _handle = h
        self._h = _handle
        self.dim, self.L, self.size, self.precision = dim, L, size, precision
        self.n_sites = L ** dim
        self.n_links = self.n_sites * dim

    # ---- lifetime
    def close(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.lq_state_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def clone(self):
        h = _vp()
        _check(load().lq_state_clone(self._h, ctypes.byref(h)), "lq_state_clone")
        return State(self.dim, self.L, self.size, self.beta, self.precision, _handle=h)

    def save(self):
        """the whole state as a checkpoint image (bytes): header, then the device fields as stored"""
        n = ctypes.c_size_t()
        _check(load().lq_state_checkpoint_bytes(self._h, ctypes.byref(n)), "lq_state_checkpoint_bytes")
        buf = ctypes.create_string_buffer(n.value)
        _check(load().lq_state_save(self._h, buf, n.value), "lq_state_save")
        return buf.raw

    @classmethod
    def load(cls, image):
        """a new state from a checkpoint image of State.save"""
        image = bytes(image)
        h = _vp()
        _check(load().lq_state_load(image, len(image), ctypes.byref(h)), "lq_state_load")
        s = cls.__new__(cls)
        s._h = h
        info = s.info()
        s.dim, s.L, s.size, s.precision = info["dim"], info["L"], info["size"], info["precision"]
        s.n_sites = s.L ** s.dim
        s.n_links = s.n_sites * s.dim
        return s

    def set_stream(self, stream_ptr):
        _check(load().lq_state_set_stream(self._h, _vp(stream_ptr)), "lq_state_set_stream")

    def set_projection_graph(self, enable):
        """Gauss projection as one graph launch (True, the default) or host-driven launches."""
        _check(load().lq_state_set_projection_graph(self._h, 1 if enable else 0), "lq_state_set_projection_graph")

    def info(self):
        d, L, pr, leap = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        size, beta = ctypes.c_double(), ctypes.c_double()
        n, t = ctypes.c_longlong(), ctypes.c_longlong()
        _check(load().lq_state_info(self._h, ctypes.byref(d), ctypes.byref(L), ctypes.byref(size), ctypes.byref(beta),
                                    ctypes.byref(pr), ctypes.byref(n), ctypes.byref(t), ctypes.byref(leap)),
               "lq_state_info")
        return dict(dim=d.value, L=L.value, size=size.value, beta=beta.value, precision=pr.value, n_sites=n.value,
                    t=t.value, is_leap=bool(leap.value))

    @property
    def beta(self):
        return self.info()["beta"]

    def set_beta(self, beta):
        _check(load().lq_state_set_beta(self._h, beta), "lq_state_set_beta")

    def set_link_update(self, link_update):
        _check(load().lq_state_set_link_update(self._h, link_update), "lq_state_set_link_update")

    @property
    def t(self):
        return self.info()["t"]

    def device_bytes(self):
        b = ctypes.c_size_t()
        _check(load().lq_state_device_bytes(self._h, ctypes.byref(b)), "lq_state_device_bytes")
        return b.value

    # ---- fields
    def set_link_matrix(self, links):
        a = np.ascontiguousarray(links, dtype=np.float64)
        _check(load().lq_links_upload(self._h, _p(a), a.size), "lq_links_upload")

    def link_matrix(self):
        out = np.empty((self.n_links, 18))
        _check(load().lq_links_download(self._h, _p(out), out.size), "lq_links_download")
        return out

    def set_links_cold(self):
        _check(load().lq_links_set_cold(self._h), "lq_links_set_cold")

    def set_links_random(self, seed):
        _check(load().lq_links_random(self._h, seed), "lq_links_random")

    def set_e_field(self, efield):
        a = np.ascontiguousarray(efield, dtype=np.float64)
        _check(load().lq_efield_upload(self._h, _p(a), a.size), "lq_efield_upload")

    def e_field(self):
        out = np.empty((self.n_sites, self.dim, 8))
        _check(load().lq_efield_download(self._h, _p(out), out.size), "lq_efield_download")
        return out

    def set_e_field_cold(self):
        _check(load().lq_efield_set_cold(self._h), "lq_efield_set_cold")

    def set_e_field_normal(self, seed, counter, std_dev):
        _check(load().lq_efield_random_normal(self._h, seed, counter, std_dev), "lq_efield_random_normal")

    # ---- observables
    def _scalar(self, fn, what):
        out = ctypes.c_double()
        _check(fn(self._h, ctypes.byref(out)), what)
        return out.value

    def hamiltonian_links(self):
        return self._scalar(load().lq_hamiltonian_links, "lq_hamiltonian_links")

    def hamiltonian_efield(self):
        return self._scalar(load().lq_hamiltonian_efield, "lq_hamiltonian_efield")

    def hamiltonian_total(self):
        return self._scalar(load().lq_hamiltonian_total, "lq_hamiltonian_total")

    def gauss_sum_div(self):
        return self._scalar(load().lq_gauss_sum_div, "lq_gauss_sum_div")

    def average_trace_plaquette(self):
        re, im = ctypes.c_double(), ctypes.c_double()
        _check(load().lq_average_trace_plaquette(self._h, ctypes.byref(re), ctypes.byref(im)),
               "lq_average_trace_plaquette")
        return complex(re.value, im.value)

    def gauss(self):
        out = np.empty((self.n_sites, 8))
        _check(load().lq_gauss_download(self._h, _p(out), out.size), "lq_gauss_download")
        return out

    # ---- differentiation
    def wilson_action(self):
        return self._scalar(load().lq_wilson_action, "lq_wilson_action")

    def wilson_action_backward(self):
        out = np.empty((self.n_sites, self.dim, 8))
        _check(load().lq_wilson_action_backward(self._h, _p(out), out.size), "lq_wilson_action_backward")
        return out

    def link_rotate(self, link, generator, angle):
        _check(load().lq_link_rotate(self._h, link, generator, angle), "lq_link_rotate")

    # ---- updates
    def metropolis_sweep(self, n_update, spread, seed, sweep):
        """one checkerboard MetropolisHastingsSweep; returns (accepted updates, mean probability)"""
        acc, pm = ctypes.c_longlong(), ctypes.c_double()
        _check(load().lq_metropolis_sweep(self._h, n_update, spread, seed, sweep, ctypes.byref(acc),
                                          ctypes.byref(pm)), "lq_metropolis_sweep")
        return acc.value, pm.value

    def overrelaxation_sweep(self, method):
        """one checkerboard OverrelaxationSweepRotation (OVERRELAX_ROTATION) or
        OverrelaxationSweepReverse (OVERRELAX_REVERSE)"""
        _check(load().lq_overrelaxation_sweep(self._h, method), "lq_overrelaxation_sweep")

    def heat_bath_sweep(self, seed, sweep):
        """one checkerboard HeatBathSweep"""
        _check(load().lq_heat_bath_sweep(self._h, seed, sweep), "lq_heat_bath_sweep")

    def field_strength(self):
        """F_ij (clover) at every site for the planes i < j: float64[V, D(D-1)/2, 18]"""
        out = np.empty((self.L ** self.dim, self.dim * (self.dim - 1) // 2, 18))
        _check(load().lq_field_strength(self._h, _p(out), out.size), "lq_field_strength")
        return out

    def magnetic_field(self):
        """magnetic_field_vec at every site: float64[V, D, 18]"""
        out = np.empty((self.L ** self.dim, self.dim, 18))
        _check(load().lq_magnetic_field(self._h, _p(out), out.size), "lq_magnetic_field")
        return out

    def leapfrog_adjoint(self, dt, n_steps, checkpoint_every=0, grads=True):
        """O = <Re Tr P>/3 after n_steps symplectic steps, dO/dbeta (momenta scaled as 1/beta) and,
        with grads, dO/dU0 (complex cotangent per link, serde layout) and dO/dE0."""
        o, db, nbytes = ctypes.c_double(), ctypes.c_double(), ctypes.c_size_t()
        gl = ge = None
        args = [None, 0, None, 0]
        if grads:
            n = self.L ** self.dim * self.dim
            gl = np.empty((n, 18))
            ge = np.empty((self.L ** self.dim, self.dim, 8))
            args = [_p(gl), gl.size, _p(ge), ge.size]
        _check(load().lq_leapfrog_adjoint(self._h, dt, n_steps, checkpoint_every, ctypes.byref(o), ctypes.byref(db),
                                          *args, ctypes.byref(nbytes)), "lq_leapfrog_adjoint")
        return dict(objective=o.value, d_objective_d_beta=db.value, grad_links=gl, grad_efield=ge,
                    work_bytes=nbytes.value)

    def project_to_gauss(self, max_steps=100000):
        steps = ctypes.c_int()
        _check(load().lq_project_gauss(self._h, max_steps, ctypes.byref(steps)), "lq_project_gauss")
        return steps.value

    def normalize_link_matrices(self):
        _check(load().lq_normalize_link_matrices(self._h), "lq_normalize_link_matrices")

    def integrate(self, mode, dt, n=1):
        _check(load().lq_integrate(self._h, mode, dt, n), "lq_integrate")

    def simulate_using_leapfrog_n(self, dt, n):
        _check(load().lq_leapfrog_n(self._h, dt, n), "lq_leapfrog_n")

    # ---- launch counters
    KERNEL_CLASSES = ("md", "gauss", "gauss_sweep", "plaquette", "reduce", "other")

    def profile_enable(self, on=True):
        _check(load().lq_profile_enable(self._h, 1 if on else 0), "lq_profile_enable")

    def profile_classes(self, names=None):
        """time only these kernel classes (names from KERNEL_CLASSES; None: all)"""
        mask = 0xFFFFFFFF if names is None else sum(1 << self.KERNEL_CLASSES.index(n) for n in names)
        _check(load().lq_profile_classes(self._h, mask), "lq_profile_classes")

    def profile_read(self, reset=False):
        """{class: (launches, total_ms)} since the last reset."""
        out = {}
        for i, name in enumerate(self.KERNEL_CLASSES):
            n, ms = ctypes.c_longlong(), ctypes.c_double()
            last = reset and i == len(self.KERNEL_CLASSES) - 1
            _check(load().lq_profile_read(self._h, i, ctypes.byref(n), ctypes.byref(ms), 1 if last else 0),
                   "lq_profile_read")
            out[name] = (n.value, ms.value)
        return out

    # ---- HMC
    def hmc_refresh(self, seed, counter, max_gauss_steps=100000):
        steps = ctypes.c_int()
        _check(load().lq_hmc_refresh(self._h, seed, counter, max_gauss_steps, ctypes.byref(steps)), "lq_hmc_refresh")
        return steps.value

    def hmc_refresh_upload(self, efield_raw, max_gauss_steps=100000):
        a = np.ascontiguousarray(efield_raw, dtype=np.float64)
        steps = ctypes.c_int()
        _check(load().lq_hmc_refresh_upload(self._h, _p(a), a.size, max_gauss_steps, ctypes.byref(steps)),
               "lq_hmc_refresh_upload")
        return steps.value

    def efield_prefetch(self, efield_raw):
        """start copying the next trajectory's raw momenta (keep the array alive and unchanged until
        hmc_refresh_prefetched returns; pinned memory makes the copy asynchronous)"""
        a = efield_raw
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise TypeError("expected a C-contiguous float64 array")
        self._prefetched = a
        _check(load().lq_efield_prefetch(self._h, _p(a), a.size), "lq_efield_prefetch")

    def hmc_refresh_prefetched(self, max_gauss_steps=100000):
        steps = ctypes.c_int()
        _check(load().lq_hmc_refresh_prefetched(self._h, max_gauss_steps, ctypes.byref(steps)),
               "lq_hmc_refresh_prefetched")
        self._prefetched = None
        return steps.value

    def hmc_propose(self, dt, n_steps):
        p, h0, h1 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(load().lq_hmc_propose(self._h, dt, n_steps, ctypes.byref(p), ctypes.byref(h0), ctypes.byref(h1)),
               "lq_hmc_propose")
        return p.value, h0.value, h1.value

    def hmc_decide(self, accept):
        _check(load().lq_hmc_decide(self._h, 1 if accept else 0), "lq_hmc_decide")

    def hmc_trajectory(self, dt, n_steps, seed, counter, uniform, max_gauss_steps=100000):
        acc, steps = ctypes.c_int(), ctypes.c_int()
        p, dh = ctypes.c_double(), ctypes.c_double()
        _check(load().lq_hmc_trajectory(self._h, dt, n_steps, seed, counter, uniform, max_gauss_steps,
                                        ctypes.byref(acc), ctypes.byref(p), ctypes.byref(dh), ctypes.byref(steps)),
               "lq_hmc_trajectory")
        return dict(accepted=bool(acc.value), prob=p.value, delta_h=dh.value, gauss_steps=steps.value)


class Batch:
    """Independent HMC ensembles of uneven side length and beta in one set of device arrays
    (lq_batch_*): every kernel of a trajectory covers all ensembles, and a trajectory can be
    replayed as one captured CUDA graph."""

    def __init__(self, dim, Ls, sizes, betas, precision=PRECISION_MIXED):
        lib = load()
        n = len(Ls)
        if len(sizes) != n or len(betas) != n:
            raise ValueError("Ls, sizes and betas must have the same length")
        self.Ls = np.ascontiguousarray(Ls, dtype=np.int32)
        sz = np.ascontiguousarray(sizes, dtype=np.float64)
        bt = np.ascontiguousarray(betas, dtype=np.float64)
        h = _vp()
        _check(lib.lq_batch_create(dim, n, self.Ls.ctypes.data_as(_ip), _p(sz), _p(bt), precision, ctypes.byref(h)),
               "lq_batch_create")
        self._h = h
        self.dim, self.n, self.precision = dim, n, precision
        self.sizes, self.betas = sz, bt
        self.last_run = 0

    def close(self):
        if getattr(self, "_h", None):
            load().lq_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr):
        _check(load().lq_batch_set_stream(self._h, _vp(stream_ptr)), "lq_batch_set_stream")

    def info(self):
        d, n, links, nbytes = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong(), ctypes.c_size_t()
        _check(load().lq_batch_info(self._h, ctypes.byref(d), ctypes.byref(n), ctypes.byref(links),
                                    ctypes.byref(nbytes)), "lq_batch_info")
        return dict(dim=d.value, n_ensembles=n.value, total_links=links.value, device_bytes=nbytes.value)

    def set_link_update(self, link_update):
        _check(load().lq_batch_set_link_update(self._h, link_update), "lq_batch_set_link_update")

    def set_seed(self, seed, counter=0):
        _check(load().lq_batch_set_seed(self._h, seed, counter), "lq_batch_set_seed")

    def set_links_random(self, seed):
        _check(load().lq_batch_links_random(self._h, seed), "lq_batch_links_random")

    def set_link_matrix(self, e, links):
        a = np.ascontiguousarray(links, dtype=np.float64)
        _check(load().lq_batch_links_upload(self._h, e, _p(a), a.size), "lq_batch_links_upload")

    def link_matrix(self, e):
        out = np.empty((int(self.Ls[e]) ** self.dim * self.dim, 18), dtype=np.float64)
        _check(load().lq_batch_links_download(self._h, e, _p(out), out.size), "lq_batch_links_download")
        return out

    def normalize_link_matrices(self):
        _check(load().lq_batch_normalize_link_matrices(self._h), "lq_batch_normalize_link_matrices")

    def average_trace_plaquette(self):
        re, im = np.empty(self.n), np.empty(self.n)
        _check(load().lq_batch_average_trace_plaquette(self._h, _p(re), _p(im)), "lq_batch_average_trace_plaquette")
        return re + 1j * im

    def autotune(self, dt=0.01, reps=3):
        _check(load().lq_batch_autotune(self._h, dt, reps), "lq_batch_autotune")
        return self.tuning()

    def tuning(self):
        out = {}
        for cls, name in enumerate(BATCH_KERNEL_CLASSES):
            g, o, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
            _check(load().lq_batch_tuning(self._h, cls, ctypes.byref(g), ctypes.byref(o), ctypes.byref(ms)),
                   "lq_batch_tuning")
            out[name] = dict(grid=g.value, order=o.value, ms=ms.value)
        return out

    def hmc_run(self, dt, n_steps, n_trajectories, max_gauss_steps=0, graph=True, measure_plaquette=False):
        flags = (BATCH_USE_GRAPH if graph else 0) | (BATCH_MEASURE_PLAQUETTE if measure_plaquette else 0)
        _check(load().lq_batch_hmc_run(self._h, dt, n_steps, n_trajectories, max_gauss_steps, flags),
               "lq_batch_hmc_run")
        self.last_run = n_trajectories

    def hmc_results(self, first=0, count=None):
        """Per-trajectory, per-ensemble results of the last run, arrays [count, n_ensembles]."""
        count = self.last_run - first if count is None else count
        shape = (count, self.n)
        dh, p, u, pl = (np.empty(shape) for _ in range(4))
        acc, steps, st = (np.empty(shape, dtype=np.int32) for _ in range(3))
        ip = lambda a: a.ctypes.data_as(_ip)
        _check(load().lq_batch_hmc_results(self._h, first, count, _p(dh), _p(p), _p(u), ip(acc), ip(steps), ip(st),
                                           _p(pl)), "lq_batch_hmc_results")
        return dict(delta_h=dh, prob=p, uniform=u, accepted=acc.astype(bool), gauss_steps=steps, status=st,
                    plaquette=pl)

    def profile_enable(self, on=True):
        """time every launch of eager trajectories (hmc_run(graph=False)) with CUDA events"""
        _check(load().lq_batch_profile_enable(self._h, 1 if on else 0), "lq_batch_profile_enable")

    def profile_read(self, reset=False):
        """(launches, summed kernel milliseconds) of eager trajectories since the last reset"""
        n, ms = ctypes.c_longlong(), ctypes.c_double()
        _check(load().lq_batch_profile_read(self._h, ctypes.byref(n), ctypes.byref(ms), 1 if reset else 0),
               "lq_batch_profile_read")
        return n.value, ms.value

    def graph_launches(self):
        n = ctypes.c_longlong()
        _check(load().lq_batch_graph_launches(self._h, ctypes.byref(n)), "lq_batch_graph_launches")
        return n.value


def fma_peak(precision=PRECISION_F64):
    """measured multiply-add peak of the current device in FLOP/s (lq_fma_peak)"""
    v = ctypes.c_double()
    _check(load().lq_fma_peak(precision, ctypes.byref(v)), "lq_fma_peak")
    return v.value


def bounds_check(reset=True):
    """(enabled, violations, first bad index + 1) of the index checks (lq_bounds_check); enabled is
    False unless the library was built with -DLQ_BOUNDS_CHECK=1"""
    en = ctypes.c_int()
    n, first = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    _check(load().lq_bounds_check(ctypes.byref(en), ctypes.byref(n), ctypes.byref(first), int(reset)),
           "lq_bounds_check")
    return bool(en.value), n.value, first.value
