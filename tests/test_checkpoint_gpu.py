"""Whole-state checkpoint (the serde derives of src/simulation/state.rs:653-654, :1046-1047):
save -> load -> k trajectories equals k trajectories of the uninterrupted state, bitwise, for the
FP64 form and the mixed form (whose compensated lo halves the image carries)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_save_load_continues_bitwise(lqgpu_mod, precision):
    G = lqgpu_mod
    dim, L, dt, n = 4, 6, 0.01, 4
    with G.State(dim, L, 1000.0, 1.5, precision) as s:
        s.set_links_random(11)
        s.set_link_update(G.LINK_UPDATE_EXP if precision == 2 else G.LINK_UPDATE_EULER)
        for k in range(2):
            s.hmc_trajectory(dt, n, 5, k, 0.5)
        s.integrate(G.SYNC_LEAP, dt)  # a leap-frog state with a non-trivial E-field and t
        image = s.save()
        info = s.info()
        s.integrate(G.LEAP_SYNC, dt)
        ref = [s.hmc_trajectory(dt, n, 5, 10 + k, 0.3) for k in range(3)]
        ref_links, ref_e = s.link_matrix(), s.e_field()
    with G.State.load(image) as r:
        assert r.info() == info
        r.integrate(G.LEAP_SYNC, dt)
        got = [r.hmc_trajectory(dt, n, 5, 10 + k, 0.3) for k in range(3)]
        assert got == ref
        assert np.array_equal(r.link_matrix(), ref_links)
        assert np.array_equal(r.e_field(), ref_e)
        assert r.save() != image  # it moved on


def test_save_refuses_pending_proposal(lqgpu_mod):
    G = lqgpu_mod
    with G.State(3, 4, 1000.0, 1.0, 0) as s:
        s.set_links_random(2)
        s.hmc_refresh(1, 0)
        s.hmc_propose(0.01, 2)
        with pytest.raises(G.LqError) as e:
            s.save()
        assert e.value.code == G.LQ_ERR_INVALID_ARGUMENT
        s.hmc_decide(True)
        assert len(s.save()) > 112
