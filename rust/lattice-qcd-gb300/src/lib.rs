//! The reference crate's state, integrator and HMC traits for device-resident states of liblqgpu.
//!
//! * [`LatticeStateGpu`] — links on the device; `LatticeState` + `LatticeStateNew` + `Clone`, the place of
//!   `LatticeStateDefault<D>` (src/simulation/state.rs:52-154, :655-850).
//! * [`LatticeStateGpuEField`] — links and E-field on the device; `LatticeStateWithEField` +
//!   `LatticeStateWithEFieldNew` + `SimulationStateSynchronous`, the place of
//!   `LatticeStateEFSyncDefault<LatticeStateDefault<D>, D>` (:165-278, :1048-1449).  Its leap-frog form is
//!   the reference's own `SimulationStateLeap<LatticeStateGpuEField<D>, D>`.
//! * [`SymplecticEulerGpu`] — the five `SymplecticIntegrator` methods (src/integrator/mod.rs:93-208) on the
//!   device, the place of `SymplecticEulerRayon`.
//! * [`HybridMonteCarloGpu`] — a `MonteCarlo` implementation with the control flow of
//!   `HybridMonteCarloDiagnostic::next_element` (src/simulation/monte_carlo/hybrid_monte_carlo.rs:465-471,
//!   :584-613): `state.monte_carlo_step(&mut hmc)` keeps its shape.
//!
//! `HybridMonteCarloDiagnostic` itself cannot drive a state of a downstream crate: it requires
//! `LatticeStateEFSyncDefault<State, D>: LatticeStateWithEField<D>`, which the reference implements only
//! for `State = LatticeStateDefault<D>`, and the orphan rule forbids implementing the reference's trait for
//! the reference's type from outside the reference crate.  Hence the separate `MonteCarlo` type.
//!
//! The `&LinkMatrix` / `&EField<D>` getters of the traits return host mirrors filled from the device on
//! first use and cleared whenever the device data changes.

pub mod hmc;
pub mod integrator;
pub mod state;

pub use hmc::HybridMonteCarloGpu;
pub use integrator::SymplecticEulerGpu;
pub use state::{LatticeStateGpu, LatticeStateGpuEField, LqError, Precision};
