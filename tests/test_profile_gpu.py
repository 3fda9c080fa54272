"""The per-class launch profile (lq_profile_enable / lq_profile_classes / lq_profile_read): with a
class mask only the selected classes carry CUDA events and are counted."""
import pytest

pytestmark = pytest.mark.gpu


def test_profile_classes_times_only_the_selected_class(lqgpu_mod):
    G = lqgpu_mod
    nsteps = 5
    with G.State(4, 6, 1000.0, 2.0, G.PRECISION_MIXED) as s:
        s.set_links_random(3)
        s.profile_enable(True)
        s.profile_classes(["md"])
        s.profile_read(reset=True)
        s.hmc_trajectory(0.01, nsteps, 7, 0, 0.5)
        p = s.profile_read(reset=True)
        assert p["md"][0] == nsteps + 1 and p["md"][1] > 0.0
        assert all(p[k][0] == 0 for k in p if k != "md")
        s.profile_classes(None)
        s.hmc_trajectory(0.01, nsteps, 7, 1, 0.5)
        p = s.profile_read(reset=True)
        assert p["md"][0] == nsteps + 1
        assert p["gauss_sweep"][0] > 0 and p["plaquette"][0] > 0
        s.profile_enable(False)
