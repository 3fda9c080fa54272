"""Failure handling on the GPU without a GPU fault: a state larger than the device's memory is refused
with LQ_ERR_OUT_OF_MEMORY by cudaMalloc on the host side (no kernel runs), everything allocated for
it is released, and the context stays usable for the next state."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_out_of_memory_is_a_status_and_the_context_survives(lqgpu_mod):
    G = lqgpu_mod
    lib = G.load()
    h = ctypes.c_void_p()
    # FP64 128^4: three link buffers of 155 GB each, beyond the GB300's 288 GB of HBM
    rc = lib.lq_state_create(4, 128, 1000.0, 1.0, G.PRECISION_F64, ctypes.byref(h))
    assert rc == G.LQ_ERR_OUT_OF_MEMORY, G.STATUS.get(rc, rc)
    assert not h.value
    assert b"cudaErrorMemoryAllocation" in lib.lq_last_error_string()
    with G.State(4, 4, 1000.0, 1.0, G.PRECISION_F64) as s:
        s.set_links_random(1)
        s.hmc_trajectory(0.01, 2, 1, 0, 0.5)
        assert 0.0 < s.hamiltonian_links() < 2.0 * 256 * 6  # sum of (1 - Re Tr P / 3) over 1536 plaquettes
