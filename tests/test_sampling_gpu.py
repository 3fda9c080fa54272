"""Two samplers of the Wilson measure exp(-beta sum (1 - Re Tr P / 3)) on the device must agree on
the average plaquette: checkerboard Metropolis (lq_metropolis_sweep) and standard HMC built from this
library's molecular dynamics and accept step (momenta N(0, 1/sqrt(beta)) from the kinetic term of
the reference's Hamiltonian, exponential link update).  D = 4, 4^4, beta 2, random start; the
tolerance is 5 standard errors estimated from 20 blocks of each chain.  A statistical check with
fixed seeds: the chains are deterministic for a given build."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def mean_err(x, blocks=20):
    x = np.asarray(x)
    b = x[: len(x) // blocks * blocks].reshape(blocks, -1).mean(axis=1)
    return x.mean(), b.std(ddof=1) / np.sqrt(blocks)


def test_standard_hmc_and_metropolis_sample_the_same_measure(lqgpu_mod):
    G = lqgpu_mod
    dim, L, beta, therm, meas = 4, 4, 2.0, 150, 800
    with G.State(dim, L, 1.0, beta, G.PRECISION_F64) as s:
        s.set_links_random(3)
        plaq = []
        for k in range(therm + meas):
            s.metropolis_sweep(4, 0.3, 9, k)
            if k >= therm:
                plaq.append(s.average_trace_plaquette().real / 3.0)
        m_mh, e_mh = mean_err(plaq)
    rng = np.random.default_rng(4)
    with G.State(dim, L, 1.0, beta, G.PRECISION_F64) as s:
        s.set_links_random(3)
        s.set_link_update(G.LINK_UPDATE_EXP)
        plaq, acc = [], 0
        for k in range(therm + meas):
            s.set_e_field(rng.normal(0.0, 1.0 / np.sqrt(beta), size=(L ** dim, dim, 8)))
            p, _, _ = s.hmc_propose(0.04, 12)
            a = p >= 1.0 or rng.uniform() < p
            s.hmc_decide(a)
            if k >= therm:
                plaq.append(s.average_trace_plaquette().real / 3.0)
                acc += a
        m_hmc, e_hmc = mean_err(plaq)
    print("Metropolis %.5f(%.5f)  standard HMC %.5f(%.5f) acceptance %.2f" % (m_mh, e_mh, m_hmc, e_hmc, acc / meas))
    assert acc / meas > 0.5
    assert abs(m_hmc - m_mh) <= 5.0 * np.hypot(e_mh, e_hmc)
