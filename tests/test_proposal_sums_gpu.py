"""The HMC proposal's start Hamiltonian.  In the FP32-arithmetic forms lq_hmc_propose takes the start
momenta's sum of squares from the second row of the kinetic-difference kernel, which walks the
elements in the order and with the arithmetic of the sum-of-squares kernel behind
lq_hamiltonian_efield: H_old must equal hamiltonian_links + hamiltonian_efield of the refreshed state
exactly, in every form."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("dim,L", [(4, 6), (3, 9)])
def test_proposal_start_hamiltonian_equals_the_separate_sums(lqgpu_mod, precision, dim, L):
    G = lqgpu_mod
    with G.State(dim, L, 1000.0, 2.0, precision) as s:
        s.set_links_random(3)
        for k in range(2):
            s.hmc_refresh(5, k)
            hl, he = s.hamiltonian_links(), s.hamiltonian_efield()
            _, h0, h1 = s.hmc_propose(0.01, 4)
            assert h0 == hl + he
            s.hmc_decide(k == 0)
