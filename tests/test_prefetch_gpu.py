"""Pipelined momenta (lq_efield_prefetch + lq_hmc_refresh_prefetched) give the trajectories of the
synchronous test mode (lq_hmc_refresh_upload) bit for bit, including when the next copy is issued
while the current trajectory runs; a refresh without a prefetch reports LQ_ERR_NO_PENDING."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_prefetched_trajectories_equal_uploaded(lqgpu_mod, precision):
    G = lqgpu_mod
    dim, L, beta, dt, n = 4, 6, 2.0, 0.01, 5
    rng = np.random.default_rng(3)
    moms = [rng.normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8)) for _ in range(3)]
    res = []
    for pipelined in (False, True):
        with G.State(dim, L, 1000.0, beta, precision) as s:
            s.set_links_random(4)
            out = []
            if pipelined:
                s.efield_prefetch(moms[0])
            for k in range(3):
                if pipelined:
                    steps = s.hmc_refresh_prefetched()
                    if k + 1 < 3:
                        s.efield_prefetch(moms[k + 1])
                else:
                    steps = s.hmc_refresh_upload(moms[k])
                p, h0, h1 = s.hmc_propose(dt, n)
                s.hmc_decide(True)
                out.append((steps, h1 - h0))
            res.append((out, s.link_matrix()))
    assert res[0][0] == res[1][0]
    assert np.array_equal(res[0][1], res[1][1])


def test_refresh_without_prefetch(lqgpu_mod):
    G = lqgpu_mod
    with G.State(4, 4, 1000.0, 2.0, G.PRECISION_MIXED) as s:
        with pytest.raises(G.LqError) as e:
            s.hmc_refresh_prefetched()
        assert e.value.code == G.LQ_ERR_NO_PENDING
