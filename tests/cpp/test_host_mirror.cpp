// Exercises the C++ host interface (lattice_qcd_rs_gb300.hpp), which mirrors the reference
// crate's state, integrator and HMC types, the way the reference's own tests use them
// (src/test/mod.rs, src/test/integrator.rs).  Prints one line per check; exit status 0 when
// every check holds.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "lattice_qcd_rs_gb300.hpp"

using namespace lattice_qcd_rs_gb300;

static int failures = 0;
#define CHECK(cond)                                                                                                    \
    do {                                                                                                               \
        if (!(cond)) {                                                                                                 \
            std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond);                                                 \
            ++failures;                                                                                                \
        } else {                                                                                                       \
            std::printf("ok   %s\n", #cond);                                                                           \
        }                                                                                                              \
    } while (0)

int main() {
    // lattice_init_error (src/test/mod.rs:603-637)
    CHECK(LatticeCyclic<3>::new_(0.0, 4).error() == LQ_ERR_NON_POSITIVE_SIZE);
    CHECK(LatticeCyclic<4>::new_(-1.0, 4).error() == LQ_ERR_NON_POSITIVE_SIZE);
    CHECK(LatticeCyclic<4>::new_(NAN, 4).error() == LQ_ERR_NON_POSITIVE_SIZE);
    CHECK(LatticeCyclic<3>::new_(1.0, 1).error() == LQ_ERR_DIM_TOO_SMALL);
    CHECK(LatticeCyclic<3>::new_(1.0, 2).is_ok());

    // a cold state: H = 0, <P> = 3
    {
        auto cold = LatticeStateDefault<4>::new_cold(1.0, 2.0, 4).unwrap();
        CHECK(cold.hamiltonian_links() == 0.0);
        CHECK(cold.average_trace_plaquette().value() == Complex(3.0, 0.0));
        CHECK(cold.link_matrix().len() == 4u * 4 * 4 * 4 * 4);
    }

    // test_sim_cold (src/test/mod.rs:430-453): a cold state is unchanged by sync->leap->sync
    {
        auto s0 = LatticeStateEFSyncDefault<4>::new_e_cold(LatticeStateDefault<4>::new_cold(10.0, 0.1, 4).unwrap());
        const LinkMatrix u0 = s0.link_matrix();
        SymplecticEulerGpu integrator;
        auto leap = integrator.integrate_sync_leap(s0, 0.1).unwrap();
        auto leap2 = integrator.integrate_leap_leap(leap, 0.1).unwrap();
        auto sync = integrator.integrate_leap_sync(leap2, 0.1).unwrap();
        CHECK(sync.link_matrix().data == u0.data);
        CHECK(sync.t() == 2);
        CHECK(s0.t() == 0); // the integrator left its argument untouched
    }

    // HMC with the unchanged driver shape: new_determinist, then monte_carlo_step
    for (int precision : {LQ_PRECISION_F64, LQ_PRECISION_MIXED}) {
        auto rng = Xoshiro256PlusPlus::seed_from_u64(0);
        auto state = LatticeStateDefault<4>::new_determinist(1000.0, 1.0, 6, rng, precision).unwrap();
        HybridMonteCarloDiagnostic<4> hmc(0.01, 10, SymplecticEulerGpu{}, Xoshiro256PlusPlus::seed_from_u64(1));
        int accepted = 0;
        for (int i = 0; i < 5; ++i) {
            state = std::move(state).monte_carlo_step(hmc).unwrap();
            accepted += hmc.has_replace_last() ? 1 : 0;
            CHECK(std::fabs(hmc.delta_h_last()) < 1e-3);
            CHECK(hmc.prob_replace_last() > 0.99);
        }
        CHECK(accepted >= 4);
        const auto p = state.average_trace_plaquette().value();
        CHECK(std::fabs(p.real()) < 0.1); // random links: <Re Tr P> ~ 0
    }

    // integrator bounds in the shape of src/test/integrator.rs:9-67 on a random state
    {
        auto rng = Xoshiro256PlusPlus::seed_from_u64(0x457893f44ab067f0ULL);
        auto st = LatticeStateDefault<3>::new_determinist(1000.0, 8.0, 4, rng).unwrap();
        auto with_e = LatticeStateEFSyncDefault<3>::new_random_e_state(std::move(st), rng);
        const double h = with_e.hamiltonian_total();
        SymplecticEulerGpu integrator;
        auto next = integrator.integrate_symplectic(with_e, 1e-4).unwrap();
        CHECK(std::fabs(h - next.hamiltonian_total()) < 1e-4);
        CHECK(next.t() == 1);
    }

    // the action's backward against a central difference on one link and generator
    {
        auto rng = Xoshiro256PlusPlus::seed_from_u64(2);
        auto st = LatticeStateDefault<4>::new_determinist(1.0, 2.0, 4, rng).unwrap();
        const EField<4> g = WilsonAction<4>::backward(st);
        const long long link = 37;
        const int a = 5;
        const double eps = 1e-5;
        check(lq_link_rotate(st.raw(), link, a, eps), "rotate");
        const double sp = WilsonAction<4>::forward(st);
        check(lq_link_rotate(st.raw(), link, a, -2 * eps), "rotate");
        const double sm = WilsonAction<4>::forward(st);
        const double fd = (sp - sm) / (2 * eps);
        CHECK(std::fabs(fd - g.data[(std::size_t)link * 8 + a]) < 1e-4);
    }

    // clover observables on a cold lattice: F = 0 and B = 0 (src/field.rs:1579-1600)
    {
        auto cold = LatticeStateDefault<3>::new_cold(1.0, 1.0, 4).unwrap();
        const auto f = cold.field_strength();
        const auto b = cold.magnetic_field();
        CHECK(f.size() == 64u * 3 * 18);
        CHECK(b.size() == 64u * 3 * 18);
        double worst = 0.0;
        for (double x : f) worst = std::fmax(worst, std::fabs(x));
        for (double x : b) worst = std::fmax(worst, std::fabs(x));
        CHECK(worst == 0.0);
    }

    // the local sweeps through monte_carlo_step: Metropolis keeps the plaquette of a cold start
    // near 3 at beta = 8 and reports accepted updates; the argument checks of ::new
    {
        CHECK(!MetropolisHastingsSweep<>::new_(0, 0.1, Xoshiro256PlusPlus::seed_from_u64(1)).has_value());
        CHECK(!MetropolisHastingsSweep<>::new_(1, 1.0, Xoshiro256PlusPlus::seed_from_u64(1)).has_value());
        auto mh = MetropolisHastingsSweep<>::new_(1, 0.1, Xoshiro256PlusPlus::seed_from_u64(1)).value();
        auto st = LatticeStateDefault<4>::new_cold(1.0, 8.0, 4).unwrap();
        for (int i = 0; i < 3; ++i) st = std::move(st).monte_carlo_step(mh).unwrap();
        CHECK(mh.number_replace_last() > 0);
        CHECK(st.average_trace_plaquette().value().real() > 2.5);
        HeatBathSweep<> hb(Xoshiro256PlusPlus::seed_from_u64(2));
        st = std::move(st).monte_carlo_step(hb).unwrap();
        CHECK(std::isfinite(st.average_trace_plaquette().value().real()));
        auto odd = LatticeStateDefault<4>::new_cold(1.0, 8.0, 3).unwrap();
        CHECK(hb.next_element(std::move(odd)).error() == LQ_ERR_INVALID_ARGUMENT);
        // overrelaxation after the heat bath, as the reference's module example does: the link
        // Hamiltonian is conserved
        OverrelaxationSweepReverse orr;
        OverrelaxationSweepRotation orot;
        const double h = st.hamiltonian_links();
        st = std::move(st).monte_carlo_step(orr).unwrap();
        st = std::move(st).monte_carlo_step(orot).unwrap();
        CHECK(std::fabs(st.hamiltonian_links() - h) <= 1e-10 * std::fabs(h));
    }

    // HybridMethodCouple / HybridMethodVec (hybrid.rs): heat bath then overrelaxation per step, as
    // the reference's module examples pair them; the errors name the failing method
    {
        HybridMethodCouple<HeatBathSweep<>, OverrelaxationSweepReverse> couple(
            HeatBathSweep<>(Xoshiro256PlusPlus::seed_from_u64(3)), OverrelaxationSweepReverse());
        auto st = LatticeStateDefault<3>::new_cold(1.0, 8.0, 4).unwrap();
        for (int i = 0; i < 2; ++i) st = std::move(st).monte_carlo_step(couple).unwrap();
        CHECK(std::isfinite(st.average_trace_plaquette().value().real()));
        auto odd = LatticeStateDefault<3>::new_cold(1.0, 8.0, 3).unwrap();
        CHECK(couple.next_element(std::move(odd)).error() == LQ_ERR_INVALID_ARGUMENT);
        CHECK(couple.error_position() == 1);

        HybridMethodVec<3> vec;
        CHECK(vec.is_empty());
        auto st2 = LatticeStateDefault<3>::new_cold(1.0, 8.0, 4).unwrap();
        auto none = vec.next_element(std::move(st2));
        CHECK(none.error() == LQ_ERR_INVALID_ARGUMENT && vec.error_index() == -1);
        HeatBathSweep<> hb2(Xoshiro256PlusPlus::seed_from_u64(4));
        OverrelaxationSweepRotation orot2;
        vec.push_method(hb2);
        vec.push_method(orot2);
        CHECK(vec.len() == 2);
        auto st3 = LatticeStateDefault<3>::new_cold(1.0, 8.0, 4).unwrap();
        st3 = std::move(st3).monte_carlo_step(vec).unwrap();
        CHECK(std::isfinite(st3.average_trace_plaquette().value().real()));
    }

    // setter with a wrong size panics, as the reference's set_link_matrix does
    {
        auto s = LatticeStateDefault<2>::new_cold(1.0, 1.0, 4).unwrap();
        LinkMatrix bad;
        bad.data.resize(18 * 3);
        bool threw = false;
        try {
            s.set_link_matrix(bad);
        } catch (const Panic &) {
            threw = true;
        }
        CHECK(threw);
    }

    std::printf("%s (%d failures)\n", failures ? "FAILED" : "PASSED", failures);
    return failures ? 1 : 0;
}
