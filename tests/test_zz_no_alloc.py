"""The allocation-free entry point lq_plaquette_sums_noalloc, through the C ABI.

It exists for callers that cannot let the library allocate device memory (a runtime that owns all
device memory in its own pool or arena, a memory-capped MPS client, or a loop that cannot afford the
device-wide synchronisation of cudaMalloc / cudaFree).  Its sums must equal those of the allocating entry points
(lq_hamiltonian_links / lq_average_trace_plaquette on an FP64 state) to the 1e-12 relative
tolerance of the other FP64 tests, on two calls in a row that share its fixed scratch array.
This file is collected last so a failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_noalloc_plaquette_sums_match_the_state_entry_points(oracle_mod, lqgpu_mod):
    torch = pytest.importorskip("torch")
    O, G = oracle_mod, lqgpu_mod
    lib = G.load()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    for dim, L in ((4, 6), (3, 10)):
        rng = O.Rng(40 + dim)
        n_plaq = L ** dim * dim * (dim - 1) // 2
        d_out = torch.zeros(3, dtype=torch.float64, device=dev)
        for call in range(2):  # two calls in a row on the same fixed scratch array
            links = O.links_random(dim, L, rng)
            d_links = torch.from_numpy(links).to(dev)
            rc = lib.lq_plaquette_sums_noalloc(dim, L, ctypes.c_void_p(d_links.data_ptr()),
                                               ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
            assert rc == G.LQ_OK, lib.lq_last_error_string()
            torch.cuda.synchronize(dev)
            out = d_out.cpu().numpy()
            with G.State(dim, L, 1.0, 1.0, G.PRECISION_F64) as s:
                s.set_link_matrix(links)
                hu = s.hamiltonian_links()
                p = s.average_trace_plaquette()
            assert abs(out[0] - hu) <= TOL * abs(hu), (call, out[0], hu)
            assert abs(out[1] / n_plaq - p.real) <= TOL, (call, out[1] / n_plaq, p.real)
            assert abs(out[2] / n_plaq - p.imag) <= TOL, (call, out[2] / n_plaq, p.imag)
            assert abs(out[0] - O.hamiltonian_links(dim, L, 1.0, links)) <= TOL * abs(hu)


def test_noalloc_rejects_lattices_beyond_its_scratch(lqgpu_mod):
    G = lqgpu_mod
    lib = G.load()
    # 64^4 sites exceed the fixed scratch; rejected on the host before any device work
    rc = lib.lq_plaquette_sums_noalloc(4, 64, ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == G.LQ_ERR_INVALID_ARGUMENT
    assert b"8388608" in lib.lq_last_error_string()
    assert lib.lq_plaquette_sums_noalloc(5, 4, ctypes.c_void_p(16), ctypes.c_void_p(16), None) == \
        G.LQ_ERR_UNSUPPORTED_DIM
    assert lib.lq_plaquette_sums_noalloc(4, 4, None, None, None) == G.LQ_ERR_INVALID_ARGUMENT
