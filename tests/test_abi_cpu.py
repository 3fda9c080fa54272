"""C ABI surface checks that need no GPU: the library builds and loads, every entry point
declared in include/lqgpu.h is exported and bound, and without a device the library
fails loudly instead of falling back to the CPU."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "lqgpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lq_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("lq_state_create", "lq_integrate", "lq_hmc_trajectory", "lq_project_gauss",
                     "lq_hamiltonian_links", "lq_average_trace_plaquette", "lq_normalize_link_matrices"):
        assert required in names


def test_library_exports_every_declared_symbol(lqgpu_mod):
    lib = lqgpu_mod.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    # and the binding knows every one of them (signatures are set, none forgotten)
    assert set(declared_functions()) == set(lqgpu_mod.SIGNATURES)


def test_dynamic_symbol_table(lqgpu_mod):
    out = subprocess.run(["nm", "-D", "--defined-only", lqgpu_mod.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (lq_[a-z0-9_]+)\b", out))
    assert set(declared_functions()) <= exported


def test_status_strings(lqgpu_mod):
    lib = lqgpu_mod.load()
    assert lib.lq_status_string(0) == b"ok"
    assert b"dimension" in lib.lq_status_string(lqgpu_mod.LQ_ERR_UNSUPPORTED_DIM)
    assert lib.lq_version() >= 100


def test_index_checks_are_off_in_the_product_build(lqgpu_mod):
    """the product library is built without the index checks: lq_bounds_check reports them off and
    makes no device call (it answers on a host without a GPU)"""
    assert lqgpu_mod.bounds_check() == (False, 0, 0)


def test_argument_validation_precedes_device_use(lqgpu_mod):
    """LatticeCyclic::new validation order (src/lattice.rs:190-201) is checked on the host
    before any device call."""
    lib = lqgpu_mod.load()
    h = ctypes.c_void_p()
    assert lib.lq_state_create(0, 4, 1.0, 1.0, 0, ctypes.byref(h)) == lqgpu_mod.LQ_ERR_ZERO_DIMENSION
    assert lib.lq_state_create(4, 4, 0.0, 1.0, 0, ctypes.byref(h)) == lqgpu_mod.LQ_ERR_NON_POSITIVE_SIZE
    assert lib.lq_state_create(4, 4, float("nan"), 1.0, 0, ctypes.byref(h)) == lqgpu_mod.LQ_ERR_NON_POSITIVE_SIZE
    assert lib.lq_state_create(4, 4, float("inf"), 1.0, 0, ctypes.byref(h)) == lqgpu_mod.LQ_ERR_NON_POSITIVE_SIZE
    assert lib.lq_state_create(3, 1, 1.0, 1.0, 0, ctypes.byref(h)) == lqgpu_mod.LQ_ERR_DIM_TOO_SMALL
    assert lib.lq_state_create(5, 4, 1.0, 1.0, 0, ctypes.byref(h)) == lqgpu_mod.LQ_ERR_UNSUPPORTED_DIM
    assert lib.lq_state_create(1, 4, 1.0, 1.0, 0, ctypes.byref(h)) == lqgpu_mod.LQ_ERR_UNSUPPORTED_DIM
    assert lib.lq_state_create(4, 4, 1.0, 1.0, 7, ctypes.byref(h)) == lqgpu_mod.LQ_ERR_INVALID_ARGUMENT
    assert lib.lq_state_create(4, 4, 1.0, 1.0, 0, None) == lqgpu_mod.LQ_ERR_INVALID_ARGUMENT
    # null handles are rejected, never dereferenced
    assert lib.lq_integrate(None, 4, 0.1, 1) == lqgpu_mod.LQ_ERR_INVALID_ARGUMENT
    assert lib.lq_hmc_decide(None, 1) == lqgpu_mod.LQ_ERR_INVALID_ARGUMENT


def test_no_cpu_fallback_without_device(lqgpu_mod):
    lib = lqgpu_mod.load()
    h = ctypes.c_void_p()
    rc = lib.lq_state_create(2, 4, 1.0, 1.0, 0, ctypes.byref(h))
    if rc == lqgpu_mod.LQ_OK:
        lib.lq_state_destroy(h)
        pytest.skip("a CUDA device is visible; the no-device path is not reachable here")
    assert rc == lqgpu_mod.LQ_ERR_NO_DEVICE
    with pytest.raises(lqgpu_mod.LqError):
        lqgpu_mod.State(2, 4)


def test_batch_argument_validation_precedes_device_use(lqgpu_mod):
    """lq_batch_create checks every ensemble as lq_state_create checks one lattice (plus the
    momentum distribution N(0, 0.5/beta) per ensemble) before any device call."""
    G = lqgpu_mod
    lib = G.load()
    h = ctypes.c_void_p()

    def create(dim, Ls, sizes, betas, precision=1):
        n = len(Ls)
        L = (ctypes.c_int * n)(*Ls)
        sz = (ctypes.c_double * n)(*sizes)
        bt = (ctypes.c_double * n)(*betas)
        return lib.lq_batch_create(dim, n, ctypes.cast(L, G._ip), ctypes.cast(sz, G._dp), ctypes.cast(bt, G._dp),
                                   precision, ctypes.byref(h))

    assert create(0, [4, 4], [1.0, 1.0], [1.0, 1.0]) == G.LQ_ERR_ZERO_DIMENSION
    assert create(4, [4, 4], [1.0, 0.0], [1.0, 1.0]) == G.LQ_ERR_NON_POSITIVE_SIZE
    assert create(4, [4, 1], [1.0, 1.0], [1.0, 1.0]) == G.LQ_ERR_DIM_TOO_SMALL
    assert create(5, [4, 4], [1.0, 1.0], [1.0, 1.0]) == G.LQ_ERR_UNSUPPORTED_DIM
    assert create(4, [4, 4], [1.0, 1.0], [1.0, 0.0]) == G.LQ_ERR_INVALID_NORMAL
    assert create(4, [4, 4], [1.0, 1.0], [1.0, -1.0]) == G.LQ_ERR_INVALID_NORMAL
    assert create(4, [4, 4], [1.0, 1.0], [1.0, 1.0], precision=7) == G.LQ_ERR_INVALID_ARGUMENT
    assert lib.lq_batch_create(4, 0, None, None, None, 1, ctypes.byref(h)) == G.LQ_ERR_INVALID_ARGUMENT
    assert lib.lq_batch_hmc_run(None, 0.1, 1, 1, 0, 1) == G.LQ_ERR_INVALID_ARGUMENT
    assert lib.lq_batch_destroy(None) == G.LQ_OK


def _param_counts(src, pattern):
    counts = {}
    for m in re.finditer(pattern, src, flags=re.S):
        params = m.group(2).strip()
        counts[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return counts


RUST = os.path.join(REPO, "rust")


def test_bindings_declare_every_function_with_its_arity(lqgpu_mod):
    """the ctypes table and the Rust -sys crate (rust/lattice-qcd-gb300-sys/src/lib.rs) bind every function
    of the header with as many parameters"""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    c = _param_counts(src, r"\b(lq_[a-z0-9_]+)\s*\(([^)]*)\)\s*;")
    sys_src = open(os.path.join(RUST, "lattice-qcd-gb300-sys", "src", "lib.rs")).read()
    block = sys_src[sys_src.index('extern "C" {'):]
    block = block[:block.index("\n}\n")]
    rust = _param_counts(block, r"pub fn (lq_[a-z0-9_]+)\(([^)]*)\)")
    assert sorted(c) == sorted(rust), set(c) ^ set(rust)
    assert {k: c[k] for k in c} == {k: rust[k] for k in c}
    assert {k: c[k] for k in c} == {k: len(lqgpu_mod.SIGNATURES[k][1]) for k in c}


def test_checkpoint_load_validates_the_image_on_the_host(lqgpu_mod):
    """lq_state_load rejects a foreign or truncated image before any device call."""
    import struct

    G = lqgpu_mod
    lib = G.load()
    h = ctypes.c_void_p()
    assert lib.lq_state_load(None, 0, ctypes.byref(h)) == G.LQ_ERR_INVALID_ARGUMENT
    assert lib.lq_state_load(b"LQGPUCK1", 8, ctypes.byref(h)) == G.LQ_ERR_INCOMPATIBLE_SIZE
    bad = b"NOTACKPT" + bytes(104)
    assert lib.lq_state_load(bad, len(bad), ctypes.byref(h)) == G.LQ_ERR_INVALID_ARGUMENT
    # a valid header whose declared field sizes the buffer does not hold
    hdr = b"LQGPUCK1" + struct.pack("<I3i2dq4i2Q4Q", 1, 4, 4, 0, 1000.0, 1.0, 0, 0, 0, 1, 0, 4096, 2048, 0, 0, 0, 0)
    assert len(hdr) == 112
    assert lib.lq_state_load(hdr, len(hdr), ctypes.byref(h)) == G.LQ_ERR_INCOMPATIBLE_SIZE
    assert not h.value


def test_rust_sys_constants_match_the_header():
    """every enumerator of include/lqgpu.h is a constant of the -sys crate with the same value"""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    header = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(LQ_[A-Z0-9_]+)\s*=\s*(\d+)", src)}
    sys_src = open(os.path.join(RUST, "lattice-qcd-gb300-sys", "src", "lib.rs")).read()
    rust = {m.group(1): int(m.group(2)) for m in re.finditer(r"pub const (LQ_[A-Z0-9_]+): c_int = (\d+);", sys_src)}
    assert header == rust, set(header.items()) ^ set(rust.items())


def test_rust_crate_implements_the_reference_traits():
    """the safe crate implements, for its device states, the reference traits a drop-in needs
    (src/simulation/state.rs:52-278, src/integrator/mod.rs:93-208,
    src/simulation/monte_carlo/mod.rs:65-77), with every required method"""
    crate = os.path.join(RUST, "lattice-qcd-gb300", "src")
    text = {f: open(os.path.join(crate, f)).read() for f in os.listdir(crate) if f.endswith(".rs")}
    every = "\n".join(text.values())

    def impl_block(trait, ty):
        m = re.search(r"impl<[^>]*>\s+%s<[^{]*?>\s+for\s+%s\b[^{]*\{" % (trait, ty), every, flags=re.S)
        assert m, (trait, ty)
        depth, i = 1, m.end()
        while depth:
            depth += {"{": 1, "}": -1}.get(every[i], 0)
            i += 1
        return every[m.end():i]

    required = {
        ("LatticeState", "LatticeStateGpu"): ["link_matrix", "set_link_matrix", "lattice", "beta", "hamiltonian_links"],
        ("LatticeStateNew", "LatticeStateGpu"): ["new"],
        ("LatticeState", "LatticeStateGpuEField"): ["link_matrix", "set_link_matrix", "lattice", "beta",
                                                      "hamiltonian_links"],
        ("LatticeStateWithEField", "LatticeStateGpuEField"): ["e_field", "set_e_field", "t", "derivative_u",
                                                                "derivative_e", "hamiltonian_efield"],
        ("LatticeStateWithEFieldNew", "LatticeStateGpuEField"): ["new"],
        ("SymplecticIntegrator", "SymplecticEulerGpu"): ["integrate_sync_sync", "integrate_leap_leap",
                                                         "integrate_sync_leap", "integrate_leap_sync",
                                                         "integrate_symplectic"],
        ("MonteCarlo", "HybridMonteCarloGpu"): ["next_element"],
    }
    for (trait, ty), methods in required.items():
        body = impl_block(trait, ty)
        for m in methods:
            assert re.search(r"\bfn %s\b" % m, body), (trait, ty, m)
    assert re.search(r"impl<const D: usize> Clone for LatticeStateGpu<D>", every)
    assert "lq_state_clone" in text["state.rs"]
    assert re.search(r"impl<[^>]*>\s+SimulationStateSynchronous<D>\s+for\s+LatticeStateGpuEField<D>", every)
    # every mode of lq_integrate that the trait's five methods need
    for mode in ("LQ_SYNC_SYNC", "LQ_LEAP_LEAP", "LQ_SYNC_LEAP", "LQ_LEAP_SYNC", "LQ_SYMPLECTIC"):
        assert "sys::%s" % mode in text["integrator.rs"], mode
