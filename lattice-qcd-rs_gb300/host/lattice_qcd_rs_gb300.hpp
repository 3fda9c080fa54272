// lattice_qcd_rs_gb300.hpp -- C++17 host interface mirroring the reference crate's API for
// the HMC path (lattice-qcd-rs v0.2.1), implemented over the C ABI of liblqgpu.so.
//
// The reference is Rust; this header keeps its type and method names, argument meanings
// and error behaviour so that code written against
//   LatticeStateDefault<D>, LatticeStateEFSyncDefault<LatticeStateDefault<D>, D>,
//   SymplecticIntegrator (SymplecticEulerRayon) and HybridMonteCarloDiagnostic
// reads the same.  States live on the device; `link_matrix()` / `e_field()` return a host
// mirror that is filled lazily and dropped whenever the device data changes.
//
// Errors: functions that return Result<T> in the reference return lq::Result<T> here (an
// error code from include/lqgpu.h or a value); functions that panic in the reference
// throw lq::Panic.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <memory>
#include <functional>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lqgpu.h"

namespace lattice_qcd_rs_gb300 {

using Real = double;
using Complex = std::complex<double>;

// ------------------------------------------------------------------ errors
struct Panic : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Rust's Result<T, E> with E = the library status code.
template <class T> class Result {
  public:
    static Result ok(T v) { return Result(std::move(v), LQ_OK); }
    static Result err(int code) { return Result(std::nullopt, code); }
    bool is_ok() const { return code_ == LQ_OK; }
    bool is_err() const { return code_ != LQ_OK; }
    int error() const { return code_; }
    T &value() {
        if (!v_) throw Panic(std::string("called unwrap on an error: ") + lq_status_string(code_));
        return *v_;
    }
    T unwrap() { return std::move(value()); }

  private:
    Result(std::optional<T> v, int c) : v_(std::move(v)), code_(c) {}
    std::optional<T> v_;
    int code_;
};

inline void check(int code, const char *what) {
    if (code != LQ_OK) {
        std::string msg = std::string(what) + ": " + lq_status_string(code);
        if (code >= LQ_ERR_CUDA) msg += std::string(" (") + lq_last_error_string() + ")";
        throw Panic(msg);
    }
}

// ------------------------------------------------------------------ random numbers
// Xoshiro256++ (Blackman & Vigna) seeded through SplitMix64: the generator the reference's
// README uses for reproducible runs (rand_xoshiro::Xoshiro256PlusPlus::seed_from_u64).
class Xoshiro256PlusPlus {
  public:
    static Xoshiro256PlusPlus seed_from_u64(uint64_t seed) {
        Xoshiro256PlusPlus r;
        uint64_t x = seed;
        for (auto &w : r.s_) {
            uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
            w = z ^ (z >> 31);
        }
        return r;
    }
    uint64_t next_u64() {
        const uint64_t result = rotl(s_[0] + s_[3], 23) + s_[0];
        const uint64_t t = s_[1] << 17;
        s_[2] ^= s_[0];
        s_[3] ^= s_[1];
        s_[1] ^= s_[2];
        s_[0] ^= s_[3];
        s_[2] ^= t;
        s_[3] = rotl(s_[3], 45);
        return result;
    }
    // uniform in [0, 1) with 52 random mantissa bits (rand 0.8 UniformFloat)
    double gen_f64() {
        const uint64_t bits = (next_u64() >> 12) | 0x3FF0000000000000ULL;
        double v;
        static_assert(sizeof(v) == sizeof(bits), "f64");
        __builtin_memcpy(&v, &bits, sizeof(v));
        return v - 1.0;
    }

  private:
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t s_[4] = {0, 0, 0, 0};
};

// ------------------------------------------------------------------ lattice
// LatticeCyclic<D> (src/lattice.rs:36-340): geometry only; the data lives on the device.
template <int D> class LatticeCyclic {
    static_assert(D == 2 || D == 3 || D == 4, "the GB300 library is instantiated for D = 2, 3 and 4");

  public:
    // LatticeCyclic::new (src/lattice.rs:190-201)
    static Result<LatticeCyclic> new_(Real size, std::size_t dim) {
        if (size <= 0.0 || std::isnan(size) || std::isinf(size)) return Result<LatticeCyclic>::err(LQ_ERR_NON_POSITIVE_SIZE);
        if (dim < 2) return Result<LatticeCyclic>::err(LQ_ERR_DIM_TOO_SMALL);
        return Result<LatticeCyclic>::ok(LatticeCyclic(size, dim));
    }
    Real size() const { return size_; }
    std::size_t dim() const { return dim_; }
    std::size_t number_of_points() const {
        std::size_t v = 1;
        for (int i = 0; i < D; ++i) v *= dim_;
        return v;
    }
    std::size_t number_of_canonical_links_space() const { return number_of_points() * D; }

  private:
    LatticeCyclic(Real s, std::size_t d) : size_(s), dim_(d) {}
    Real size_;
    std::size_t dim_;
};

// Host copies in the reference's serde layouts.
struct LinkMatrix {
    std::vector<double> data; // [link][col][row][re,im], 18 per link
    std::size_t len() const { return data.size() / 18; }
};
template <int D> struct EField {
    std::vector<double> data; // [site][mu][8]
    std::size_t len() const { return data.size() / (8 * D); }
};

// ------------------------------------------------------------------ states
namespace detail {
struct Handle {
    lq_state *h = nullptr;
    explicit Handle(lq_state *p) : h(p) {}
    ~Handle() {
        if (h) lq_state_destroy(h);
    }
    Handle(const Handle &) = delete;
    Handle &operator=(const Handle &) = delete;
};
} // namespace detail

template <int D> class LatticeStateEFSyncDefault;

// LatticeStateDefault<D> (src/simulation/state.rs:652-850), device resident.
template <int D> class LatticeStateDefault {
  public:
    static constexpr Real CA = 3.0;

    // LatticeStateDefault::new_cold (src/simulation/state.rs:670-678)
    static Result<LatticeStateDefault> new_cold(Real size, Real beta, std::size_t number_of_points,
                                                int precision = LQ_PRECISION_F64) {
        auto lat = LatticeCyclic<D>::new_(size, number_of_points);
        if (lat.is_err()) return Result<LatticeStateDefault>::err(lat.error());
        lq_state *h = nullptr;
        const int rc = lq_state_create(D, (int)number_of_points, size, beta, precision, &h);
        if (rc) return Result<LatticeStateDefault>::err(rc);
        return Result<LatticeStateDefault>::ok(LatticeStateDefault(lat.unwrap(), beta, h));
    }

    // LatticeStateDefault::new_determinist (src/simulation/state.rs:705-714): random_su3 links;
    // the device draws them from a Philox stream keyed by one value of the caller's generator.
    template <class Rng>
    static Result<LatticeStateDefault> new_determinist(Real size, Real beta, std::size_t number_of_points, Rng &rng,
                                                       int precision = LQ_PRECISION_F64) {
        auto r = new_cold(size, beta, number_of_points, precision);
        if (r.is_err()) return r;
        LatticeStateDefault s = r.unwrap();
        const int rc = lq_links_random(s.raw(), rng.next_u64());
        if (rc) return Result<LatticeStateDefault>::err(rc);
        return Result<LatticeStateDefault>::ok(std::move(s));
    }

    // LatticeStateNew::new (src/simulation/state.rs:730-746)
    static Result<LatticeStateDefault> new_(const LatticeCyclic<D> &lattice, Real beta, const LinkMatrix &links,
                                            int precision = LQ_PRECISION_F64) {
        if (links.len() != lattice.number_of_canonical_links_space())
            return Result<LatticeStateDefault>::err(LQ_ERR_INCOMPATIBLE_SIZE);
        auto r = new_cold(lattice.size(), beta, lattice.dim(), precision);
        if (r.is_err()) return r;
        LatticeStateDefault s = r.unwrap();
        const int rc = lq_links_upload(s.raw(), links.data.data(), links.data.size());
        if (rc) return Result<LatticeStateDefault>::err(rc);
        return Result<LatticeStateDefault>::ok(std::move(s));
    }

    LatticeStateDefault(LatticeStateDefault &&) = default;
    LatticeStateDefault &operator=(LatticeStateDefault &&) = default;
    // State: Clone (device copy)
    LatticeStateDefault clone() const {
        lq_state *c = nullptr;
        check(lq_state_clone(raw(), &c), "lq_state_clone");
        return LatticeStateDefault(lattice_, beta_, c);
    }

    // LatticeState::link_matrix (src/simulation/state.rs:73)
    const LinkMatrix &link_matrix() const {
        if (!links_mirror_) {
            LinkMatrix m;
            m.data.resize(lattice_.number_of_canonical_links_space() * 18);
            check(lq_links_download(raw(), m.data.data(), m.data.size()), "lq_links_download");
            links_mirror_ = std::move(m);
        }
        return *links_mirror_;
    }
    // LatticeState::set_link_matrix (src/simulation/state.rs:808-815): panics on a size mismatch
    void set_link_matrix(const LinkMatrix &links) {
        if (links.len() != lattice_.number_of_canonical_links_space()) throw Panic("Link matrices are not of the correct size");
        check(lq_links_upload(raw(), links.data.data(), links.data.size()), "lq_links_upload");
        links_mirror_.reset();
    }
    const LatticeCyclic<D> &lattice() const { return lattice_; }
    Real beta() const { return beta_; }
    // LatticeState::hamiltonian_links (src/simulation/state.rs:821-849)
    Real hamiltonian_links() const {
        double h = 0.0;
        check(lq_hamiltonian_links(raw(), &h), "lq_hamiltonian_links");
        return h;
    }
    // LatticeState::average_trace_plaquette (src/simulation/state.rs:115-117)
    std::optional<Complex> average_trace_plaquette() const {
        double re = 0.0, im = 0.0;
        if (lq_average_trace_plaquette(raw(), &re, &im) != LQ_OK) return std::nullopt;
        return Complex(re, im);
    }
    // LinkMatrix::f_mu_nu at every point for the planes i < j (src/field.rs:822-835), computed on the
    // device: [site][plane][18], planes in the order (0,1), (0,2), ..., (D-2,D-1)
    std::vector<double> field_strength() const {
        std::vector<double> out(lattice_.number_of_points() * (std::size_t)(D * (D - 1) / 2) * 18);
        check(lq_field_strength(raw(), out.data(), out.size()), "lq_field_strength");
        return out;
    }
    // LinkMatrix::magnetic_field_vec at every point (src/field.rs:837-871): [site][k][18]
    std::vector<double> magnetic_field() const {
        std::vector<double> out(lattice_.number_of_points() * (std::size_t)D * 18);
        check(lq_magnetic_field(raw(), out.data(), out.size()), "lq_magnetic_field");
        return out;
    }
    // LatticeStateDefault::normalize_link_matrices (src/simulation/state.rs:754-756)
    void normalize_link_matrices() {
        check(lq_normalize_link_matrices(raw()), "lq_normalize_link_matrices");
        links_mirror_.reset();
    }
    // LatticeState::monte_carlo_step (src/simulation/state.rs:103-109)
    template <class M> auto monte_carlo_step(M &m) && { return m.next_element(std::move(*this)); }

    lq_state *raw() const { return handle_->h; }
    void invalidate_mirror() { links_mirror_.reset(); }

  private:
    friend class LatticeStateEFSyncDefault<D>;
    LatticeStateDefault(const LatticeCyclic<D> &l, Real beta, lq_state *h)
        : lattice_(l), beta_(beta), handle_(std::make_unique<detail::Handle>(h)) {}
    LatticeCyclic<D> lattice_;
    Real beta_;
    std::unique_ptr<detail::Handle> handle_;
    mutable std::optional<LinkMatrix> links_mirror_;
};

// LatticeStateEFSyncDefault<LatticeStateDefault<D>, D> (src/simulation/state.rs:1043-1449).
// The E-field shares the device state of the wrapped LatticeStateDefault.
template <int D> class LatticeStateEFSyncDefault {
  public:
    static constexpr Real CA = 3.0;

    // new_random_e_state (src/simulation/state.rs:1093-1108): E ~ N(0, 0.5/beta) drawn on the
    // device (Philox keyed by one value of `rng`), then project_to_gauss.  Panics like the
    // reference when beta gives no valid distribution or the projection fails.
    template <class Rng> static LatticeStateEFSyncDefault new_random_e_state(LatticeStateDefault<D> state, Rng &rng) {
        int steps = 0;
        check(lq_hmc_refresh(state.raw(), rng.next_u64(), 0, 0, &steps), "new_random_e_state");
        return LatticeStateEFSyncDefault(std::move(state), steps);
    }
    // new_e_cold (src/simulation/state.rs:1111-1120)
    static LatticeStateEFSyncDefault new_e_cold(LatticeStateDefault<D> state) {
        check(lq_efield_set_cold(state.raw()), "lq_efield_set_cold");
        return LatticeStateEFSyncDefault(std::move(state), 0);
    }
    // LatticeStateWithEFieldNew::new (src/simulation/state.rs:1342-1361)
    static Result<LatticeStateEFSyncDefault> new_(const LatticeCyclic<D> &lattice, Real beta, const EField<D> &e,
                                                  const LinkMatrix &links, std::size_t t,
                                                  int precision = LQ_PRECISION_F64) {
        if (e.len() != lattice.number_of_points()) return Result<LatticeStateEFSyncDefault>::err(LQ_ERR_INCOMPATIBLE_SIZE);
        auto st = LatticeStateDefault<D>::new_(lattice, beta, links, precision);
        if (st.is_err()) return Result<LatticeStateEFSyncDefault>::err(st.error());
        LatticeStateDefault<D> s = st.unwrap();
        const int rc = lq_efield_upload(s.raw(), e.data.data(), e.data.size());
        if (rc) return Result<LatticeStateEFSyncDefault>::err(rc);
        LatticeStateEFSyncDefault out(std::move(s), 0);
        out.t_ = t;
        return Result<LatticeStateEFSyncDefault>::ok(std::move(out));
    }

    LatticeStateEFSyncDefault(LatticeStateEFSyncDefault &&) = default;
    LatticeStateEFSyncDefault &operator=(LatticeStateEFSyncDefault &&) = default;
    LatticeStateEFSyncDefault clone() const {
        LatticeStateEFSyncDefault c(state_.clone(), gauss_steps_);
        c.t_ = t_;
        return c;
    }

    const LinkMatrix &link_matrix() const { return state_.link_matrix(); }
    void set_link_matrix(const LinkMatrix &l) { state_.set_link_matrix(l); }
    const LatticeCyclic<D> &lattice() const { return state_.lattice(); }
    Real beta() const { return state_.beta(); }
    Real hamiltonian_links() const { return state_.hamiltonian_links(); }
    std::optional<Complex> average_trace_plaquette() const { return state_.average_trace_plaquette(); }

    // LatticeStateWithEField (src/simulation/state.rs:1370-1399)
    const EField<D> &e_field() const {
        if (!e_mirror_) {
            EField<D> e;
            e.data.resize(lattice().number_of_points() * D * 8);
            check(lq_efield_download(raw(), e.data.data(), e.data.size()), "lq_efield_download");
            e_mirror_ = std::move(e);
        }
        return *e_mirror_;
    }
    void set_e_field(const EField<D> &e) {
        if (e.len() != lattice().number_of_points()) throw Panic("e_field is not of the correct size");
        check(lq_efield_upload(raw(), e.data.data(), e.data.size()), "lq_efield_upload");
        e_mirror_.reset();
    }
    std::size_t t() const { return t_; }
    Real hamiltonian_efield() const {
        double h = 0.0;
        check(lq_hamiltonian_efield(raw(), &h), "lq_hamiltonian_efield");
        return h;
    }
    Real hamiltonian_total() const { return hamiltonian_links() + hamiltonian_efield(); }
    // EField::project_to_gauss applied to this state's field (src/field.rs:1265-1294)
    int project_to_gauss(int max_steps = 0) {
        int steps = 0;
        check(lq_project_gauss(raw(), max_steps, &steps), "lq_project_gauss");
        e_mirror_.reset();
        return steps;
    }
    int gauss_steps_of_refresh() const { return gauss_steps_; }

    // LatticeStateEFSyncDefault::state_owned (src/simulation/state.rs:1065-1072)
    LatticeStateDefault<D> state_owned() && {
        state_.invalidate_mirror();
        return std::move(state_);
    }
    lq_state *raw() const { return state_.raw(); }
    void device_changed(std::size_t t) {
        t_ = t;
        state_.invalidate_mirror();
        e_mirror_.reset();
    }

  private:
    LatticeStateEFSyncDefault(LatticeStateDefault<D> s, int steps) : state_(std::move(s)), gauss_steps_(steps) {}
    LatticeStateDefault<D> state_;
    std::size_t t_ = 0;
    int gauss_steps_ = 0;
    mutable std::optional<EField<D>> e_mirror_;
};

// SimulationStateLeap<State, D> (src/simulation/state.rs:851-1040): a leap-frog state, E at
// half time steps.
template <int D> class SimulationStateLeap {
  public:
    explicit SimulationStateLeap(LatticeStateEFSyncDefault<D> s) : state_(std::move(s)) {}
    const LatticeStateEFSyncDefault<D> &state() const { return state_; }
    LatticeStateEFSyncDefault<D> &state_mut() { return state_; }
    LatticeStateEFSyncDefault<D> into_state() && { return std::move(state_); }

  private:
    LatticeStateEFSyncDefault<D> state_;
};

// ------------------------------------------------------------------ integrator
// SymplecticIntegrator implemented by the device (SymplecticEulerRayon,
// src/integrator/symplectic_euler_rayon.rs:120-252).  Like the reference, every method
// returns a new state and leaves its argument untouched (the argument is cloned on the
// device); the *_in_place variants skip the copy.
class SymplecticEulerGpu {
  public:
    template <int D>
    Result<LatticeStateEFSyncDefault<D>> integrate_sync_sync(const LatticeStateEFSyncDefault<D> &l, Real dt) const {
        return run(l.clone(), LQ_SYNC_SYNC, dt, 1);
    }
    template <int D>
    Result<SimulationStateLeap<D>> integrate_leap_leap(const SimulationStateLeap<D> &l, Real dt) const {
        auto r = run(l.state().clone(), LQ_LEAP_LEAP, dt, 1);
        if (r.is_err()) return Result<SimulationStateLeap<D>>::err(r.error());
        return Result<SimulationStateLeap<D>>::ok(SimulationStateLeap<D>(r.unwrap()));
    }
    template <int D>
    Result<SimulationStateLeap<D>> integrate_sync_leap(const LatticeStateEFSyncDefault<D> &l, Real dt) const {
        auto r = run(l.clone(), LQ_SYNC_LEAP, dt, 1);
        if (r.is_err()) return Result<SimulationStateLeap<D>>::err(r.error());
        return Result<SimulationStateLeap<D>>::ok(SimulationStateLeap<D>(r.unwrap()));
    }
    template <int D>
    Result<LatticeStateEFSyncDefault<D>> integrate_leap_sync(const SimulationStateLeap<D> &l, Real dt) const {
        return run(l.state().clone(), LQ_LEAP_SYNC, dt, 1);
    }
    template <int D>
    Result<LatticeStateEFSyncDefault<D>> integrate_symplectic(const LatticeStateEFSyncDefault<D> &l, Real dt) const {
        return run(l.clone(), LQ_SYMPLECTIC, dt, 1);
    }
    // simulate_symplectic_n (src/simulation/state.rs:470-491) on the state itself
    template <int D> int simulate_symplectic_n_in_place(LatticeStateEFSyncDefault<D> &l, Real dt, int n) const {
        const int rc = lq_integrate(l.raw(), LQ_SYMPLECTIC, dt, n);
        if (rc == LQ_OK) l.device_changed(l.t() + (std::size_t)n);
        return rc;
    }

  private:
    template <int D> static Result<LatticeStateEFSyncDefault<D>> run(LatticeStateEFSyncDefault<D> s, int mode, Real dt, int n) {
        const int rc = lq_integrate(s.raw(), mode, dt, n);
        if (rc) return Result<LatticeStateEFSyncDefault<D>>::err(rc);
        long long t = 0;
        check(lq_state_info(s.raw(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &t, nullptr), "lq_state_info");
        s.device_changed((std::size_t)t);
        return Result<LatticeStateEFSyncDefault<D>>::ok(std::move(s));
    }
};

// ------------------------------------------------------------------ differentiation
// The Wilson action as an autograd-style function: forward gives S = beta sum (1 - Re Tr P / 3),
// backward the gradient dS/dtheta^a for U -> exp(i theta^a T^a) U on every link, in the E-field
// layout.  The reference's force derivative_e (src/simulation/state.rs:1420-1448) is
// -sqrt(2 C_A)/(size beta) times the gradient.
template <int D> struct WilsonAction {
    static Real forward(const LatticeStateDefault<D> &s) {
        double v = 0.0;
        check(lq_wilson_action(s.raw(), &v), "lq_wilson_action");
        return v;
    }
    static EField<D> backward(const LatticeStateDefault<D> &s) {
        EField<D> g;
        g.data.resize(s.lattice().number_of_points() * D * 8);
        check(lq_wilson_action_backward(s.raw(), g.data.data(), g.data.size()), "lq_wilson_action_backward");
        return g;
    }
};

// ------------------------------------------------------------------ HMC driver
// HybridMonteCarloDiagnostic<LatticeStateDefault<D>, Rng, I, D>
// (src/simulation/monte_carlo/hybrid_monte_carlo.rs:302-614).  next_element draws the momenta
// (device Philox keyed by the generator), projects them, integrates, and accepts with
// Bernoulli(prob): prob == 1 accepts without drawing, otherwise one uniform u < prob.
// MetropolisHastingsSweep (src/simulation/monte_carlo/metropolis_hastings_sweep.rs) on the device:
// one next_element is one checkerboard sweep (lq_metropolis_sweep); the Philox seed of the sweeps is
// drawn from the Rng once, the sweep counter advances per call.
template <class Rng = Xoshiro256PlusPlus> class MetropolisHastingsSweep {
  public:
    // MetropolisHastingsSweep::new: None unless number_of_update >= 1 and 0 < spread < 1
    static std::optional<MetropolisHastingsSweep> new_(std::size_t number_of_update, Real spread, Rng rng) {
        if (number_of_update == 0 || !(spread > 0.0) || !(spread < 1.0)) return std::nullopt;
        return MetropolisHastingsSweep(number_of_update, spread, std::move(rng));
    }
    template <int D> Result<LatticeStateDefault<D>> next_element(LatticeStateDefault<D> state) {
        long long acc = 0;
        double pm = 0.0;
        const int rc = lq_metropolis_sweep(state.raw(), (int)n_, spread_, seed_, sweep_++, &acc, &pm);
        if (rc) return Result<LatticeStateDefault<D>>::err(rc);
        state.invalidate_mirror();
        number_replace_last_ = (std::size_t)acc;
        prob_replace_mean_ = pm;
        return Result<LatticeStateDefault<D>>::ok(std::move(state));
    }
    std::size_t number_replace_last() const { return number_replace_last_; }
    Real prob_replace_mean() const { return prob_replace_mean_; }

  private:
    MetropolisHastingsSweep(std::size_t n, Real spread, Rng rng)
        : n_(n), spread_(spread), rng_(std::move(rng)), seed_(rng_.next_u64()) {}
    std::size_t n_;
    Real spread_;
    Rng rng_;
    uint64_t seed_;
    uint64_t sweep_ = 0;
    std::size_t number_replace_last_ = 0;
    Real prob_replace_mean_ = 0.0;
};

// HeatBathSweep (src/simulation/monte_carlo/heat_bath.rs) on the device: one checkerboard sweep per
// next_element (lq_heat_bath_sweep)
template <class Rng = Xoshiro256PlusPlus> class HeatBathSweep {
  public:
    explicit HeatBathSweep(Rng rng) : rng_(std::move(rng)), seed_(rng_.next_u64()) {}
    template <int D> Result<LatticeStateDefault<D>> next_element(LatticeStateDefault<D> state) {
        const int rc = lq_heat_bath_sweep(state.raw(), seed_, sweep_++);
        if (rc) return Result<LatticeStateDefault<D>>::err(rc);
        state.invalidate_mirror();
        return Result<LatticeStateDefault<D>>::ok(std::move(state));
    }

  private:
    Rng rng_;
    uint64_t seed_;
    uint64_t sweep_ = 0;
};

// OverrelaxationSweepRotation / OverrelaxationSweepReverse (overrelaxation.rs:77-205): no random
// numbers; MonteCarlo::next_element with Error = Never in the reference (device errors here).
class OverrelaxationSweepRotation {
  public:
    template <int D> Result<LatticeStateDefault<D>> next_element(LatticeStateDefault<D> state) {
        const int rc = lq_overrelaxation_sweep(state.raw(), LQ_OVERRELAX_ROTATION);
        if (rc) return Result<LatticeStateDefault<D>>::err(rc);
        state.invalidate_mirror();
        return Result<LatticeStateDefault<D>>::ok(std::move(state));
    }
};
class OverrelaxationSweepReverse {
  public:
    template <int D> Result<LatticeStateDefault<D>> next_element(LatticeStateDefault<D> state) {
        const int rc = lq_overrelaxation_sweep(state.raw(), LQ_OVERRELAX_REVERSE);
        if (rc) return Result<LatticeStateDefault<D>>::err(rc);
        state.invalidate_mirror();
        return Result<LatticeStateDefault<D>>::ok(std::move(state));
    }
};

// HybridMethodCouple (src/simulation/monte_carlo/hybrid.rs:327-420): the first method, then the
// second, on each step.  An error stops the step; error_position() tells which method raised it
// (1: HybridMethodCoupleError::ErrorFirst, 2: ErrorSecond).
template <class MC1, class MC2> class HybridMethodCouple {
  public:
    HybridMethodCouple(MC1 first, MC2 second) : first_(std::move(first)), second_(std::move(second)) {}
    template <int D> Result<LatticeStateDefault<D>> next_element(LatticeStateDefault<D> state) {
        error_position_ = 0;
        auto r1 = first_.next_element(std::move(state));
        if (r1.is_err()) {
            error_position_ = 1;
            return r1;
        }
        auto r2 = second_.next_element(r1.unwrap());
        if (r2.is_err()) error_position_ = 2;
        return r2;
    }
    int error_position() const { return error_position_; }
    MC1 &first() { return first_; }
    MC2 &second() { return second_; }

  private:
    MC1 first_;
    MC2 second_;
    int error_position_ = 0;
};

// HybridMethodVec (hybrid.rs:156-270): the referenced methods in order on each step (the reference
// holds `&mut dyn MonteCarlo`; the caller keeps the methods alive here too).  No method: the
// HybridMethodVecError::NoMethod case, LQ_ERR_INVALID_ARGUMENT with error_index() = -1; an error of
// method i stops the step with error_index() = i (HybridMethodVecError::Error(i, e)).
template <int D> class HybridMethodVec {
  public:
    using State = LatticeStateDefault<D>;
    template <class M> void push_method(M &m) {
        methods_.push_back([&m](State s) { return m.next_element(std::move(s)); });
    }
    void pop_method() {
        if (!methods_.empty()) methods_.pop_back();
    }
    std::size_t len() const { return methods_.size(); }
    bool is_empty() const { return methods_.empty(); }
    Result<State> next_element(State state) {
        error_index_ = -1;
        if (methods_.empty()) return Result<State>::err(LQ_ERR_INVALID_ARGUMENT);
        for (std::size_t i = 0; i < methods_.size(); ++i) {
            auto r = methods_[i](std::move(state));
            if (r.is_err()) {
                error_index_ = (int)i;
                return r;
            }
            state = r.unwrap();
        }
        return Result<State>::ok(std::move(state));
    }
    int error_index() const { return error_index_; }

  private:
    std::vector<std::function<Result<State>(State)>> methods_;
    int error_index_ = -1;
};

template <int D, class Rng = Xoshiro256PlusPlus, class I = SymplecticEulerGpu> class HybridMonteCarloDiagnostic {
  public:
    HybridMonteCarloDiagnostic(Real delta_t, std::size_t number_of_steps, I integrator, Rng rng)
        : delta_t_(delta_t), n_(number_of_steps), integrator_(std::move(integrator)), rng_(std::move(rng)) {}

    // MonteCarlo::next_element (hybrid_monte_carlo.rs:465-471); errors: MultiIntegrationError
    // (LQ_ERR_ZERO_INTEGRATION) and device errors.
    Result<LatticeStateDefault<D>> next_element(LatticeStateDefault<D> state) {
        if (n_ == 0) return Result<LatticeStateDefault<D>>::err(LQ_ERR_ZERO_INTEGRATION);
        auto with_e = LatticeStateEFSyncDefault<D>::new_random_e_state(std::move(state), rng_);
        double p = 0.0, h0 = 0.0, h1 = 0.0;
        int rc = lq_hmc_propose(with_e.raw(), delta_t_, (int)n_, &p, &h0, &h1);
        if (rc) return Result<LatticeStateDefault<D>>::err(rc);
        bool accept = true;
        if (!(p >= 1.0)) accept = rng_.gen_f64() < p;
        rc = lq_hmc_decide(with_e.raw(), accept ? 1 : 0);
        if (rc) return Result<LatticeStateDefault<D>>::err(rc);
        prob_replace_last_ = p;
        has_replace_last_ = accept;
        last_delta_h_ = h1 - h0;
        return Result<LatticeStateDefault<D>>::ok(std::move(with_e).state_owned());
    }
    Real prob_replace_last() const { return prob_replace_last_; }
    bool has_replace_last() const { return has_replace_last_; }
    Real delta_h_last() const { return last_delta_h_; }
    Real delta_t() const { return delta_t_; }
    std::size_t number_of_steps() const { return n_; }
    const I &integrator() const { return integrator_; }
    Rng &rng_mut() { return rng_; }

  private:
    Real delta_t_;
    std::size_t n_;
    I integrator_;
    Rng rng_;
    Real prob_replace_last_ = 0.0;
    bool has_replace_last_ = false;
    Real last_delta_h_ = 0.0;
};

} // namespace lattice_qcd_rs_gb300
