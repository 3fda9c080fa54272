// hmc_driver_timing.cpp -- wall-clock throughput of the C++ host interface's
// HybridMonteCarloDiagnostic driving a device-resident state, the way a program written against the
// reference (src/simulation/monte_carlo/hybrid_monte_carlo.rs:465-471) runs it: new_determinist, then
// monte_carlo_step in a loop (momenta from the device generator keyed by the driver's Xoshiro256++,
// the accept decision on the host from the proposal's probability).
//
//   hmc_driver_timing L trajectories warmup precision md_steps dt beta
//
// Prints one JSON object: link-updates per second over the timed trajectories (host clock; every
// trajectory ends with the host reading its proposal back, and the timed region ends with a read of
// the plaquette).
#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "lattice_qcd_rs_gb300.hpp"

using namespace lattice_qcd_rs_gb300;

int main(int argc, char **argv) {
    if (argc != 8) {
        std::fprintf(stderr, "usage: %s L trajectories warmup precision md_steps dt beta\n", argv[0]);
        return 2;
    }
    const int L = std::atoi(argv[1]), n = std::atoi(argv[2]), warmup = std::atoi(argv[3]);
    const int precision = std::atoi(argv[4]), md_steps = std::atoi(argv[5]);
    const double dt = std::atof(argv[6]), beta = std::atof(argv[7]);
    if (L < 2 || n < 1 || warmup < 0 || md_steps < 1) return 2;
    auto rng = Xoshiro256PlusPlus::seed_from_u64(1);
    auto made = LatticeStateDefault<4>::new_determinist(1000.0, beta, (std::size_t)L, rng, precision);
    if (made.is_err()) {
        std::fprintf(stderr, "state: error %d\n", made.error());
        return 1;
    }
    auto state = made.unwrap();
    HybridMonteCarloDiagnostic<4> hmc(dt, (std::size_t)md_steps, SymplecticEulerGpu{},
                                      Xoshiro256PlusPlus::seed_from_u64(2));
    int accepted = 0;
    auto step = [&]() -> bool {
        auto r = std::move(state).monte_carlo_step(hmc);
        if (r.is_err()) {
            std::fprintf(stderr, "monte_carlo_step: error %d\n", r.error());
            return false;
        }
        state = r.unwrap();
        accepted += hmc.has_replace_last() ? 1 : 0;
        return true;
    };
    for (int i = 0; i < warmup; ++i)
        if (!step()) return 1;
    accepted = 0;
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < n; ++i)
        if (!step()) return 1;
    const auto plaquette = state.average_trace_plaquette();
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (!plaquette) return 1;
    const double links = 1.0 * L * L * L * L * 4;
    std::printf("{\"value\": %.6e, \"unit\": \"link-updates/s\", \"ms_per_trajectory\": %.4f, \"trajectories\": %d, "
                "\"accepted\": %d, \"plaquette\": %.12f}\n",
                links * md_steps * n / s, 1000.0 * s / n, n, accepted, plaquette->real() / 3.0);
    return 0;
}
