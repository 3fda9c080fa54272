//! The HMC step on the device with the control flow of `HybridMonteCarloDiagnostic::next_element`
//! (src/simulation/monte_carlo/hybrid_monte_carlo.rs:465-471, :584-613): refresh the momenta
//! (N(0, 0.5/beta), projected to the Gauss law), integrate `number_of_steps` symplectic steps, accept
//! with probability min(1, exp(H_old - H_new)) by the reference's Bernoulli rule.  The momenta are drawn
//! on the device from a Philox stream keyed by a seed the caller's rng provides, so no field crosses
//! the bus; the accept uniform comes from the caller's rng.
use lattice_qcd_gb300_sys as sys;
use lattice_qcd_rs::simulation::MonteCarlo;
use lattice_qcd_rs::Real;
use std::os::raw::c_int;

use crate::state::{check, LatticeStateGpu, LqError};

pub struct HybridMonteCarloGpu<Rng: rand::Rng> {
    delta_t: Real,
    number_of_steps: usize,
    rng: Rng,
    seed: u64,
    counter: u64,
    /// 0 lets the device loop stop after its default limit of 10001 projection sweeps
    max_gauss_steps: c_int,
    prob_replace_last: Real,
    has_replace_last: bool,
    gauss_steps_last: c_int,
}

impl<Rng: rand::Rng> HybridMonteCarloGpu<Rng> {
    /// `HybridMonteCarloDiagnostic::new(delta_t, number_of_steps, integrator, rng)`: the device integrator
    /// is implied
    pub fn new(delta_t: Real, number_of_steps: usize, mut rng: Rng) -> Self {
        let seed = rng.next_u64();
        Self {
            delta_t,
            number_of_steps,
            rng,
            seed,
            counter: 0,
            max_gauss_steps: 0,
            prob_replace_last: 0.0,
            has_replace_last: false,
            gauss_steps_last: 0,
        }
    }
    pub const fn prob_replace_last(&self) -> Real {
        self.prob_replace_last
    }
    pub const fn has_replace_last(&self) -> bool {
        self.has_replace_last
    }
    /// projection sweeps of the last refresh
    pub const fn gauss_steps_last(&self) -> c_int {
        self.gauss_steps_last
    }
    pub fn rng_mut(&mut self) -> &mut Rng {
        &mut self.rng
    }
}

impl<Rng: rand::Rng, const D: usize> MonteCarlo<LatticeStateGpu<D>, D> for HybridMonteCarloGpu<Rng> {
    type Error = LqError;

    fn next_element(&mut self, mut state: LatticeStateGpu<D>) -> Result<LatticeStateGpu<D>, LqError> {
        let s = state.as_raw();
        let mut steps: c_int = 0;
        check(unsafe { sys::lq_hmc_refresh(s, self.seed, self.counter, self.max_gauss_steps, &mut steps) })?;
        self.counter += 1;
        self.gauss_steps_last = steps;
        let (mut prob, mut h_old, mut h_new) = (0.0, 0.0, 0.0);
        check(unsafe { sys::lq_hmc_propose(s, self.delta_t, self.number_of_steps as c_int, &mut prob, &mut h_old, &mut h_new) })?;
        // rand 0.8's Bernoulli: p = 1 always accepts without a draw, otherwise one uniform < p
        let accept = prob >= 1.0 || self.rng.gen::<f64>() < prob;
        check(unsafe { sys::lq_hmc_decide(s, accept as c_int) })?;
        self.prob_replace_last = prob;
        self.has_replace_last = accept;
        state.invalidate();
        Ok(state)
    }
}
