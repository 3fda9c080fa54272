//! The device integrator: the five methods of `SymplecticIntegrator` (src/integrator/mod.rs:93-208) with
//! `SymplecticEulerRayon`'s arithmetic (src/integrator/symplectic_euler_rayon.rs:120-252), run by
//! `lq_integrate` on a device copy of the state.
use lattice_qcd_gb300_sys as sys;
use lattice_qcd_rs::lattice::{Direction, DirectionList};
use lattice_qcd_rs::simulation::SimulationStateLeap;
use lattice_qcd_rs::integrator::SymplecticIntegrator;
use lattice_qcd_rs::Real;
use std::os::raw::c_int;

use crate::state::{check, LatticeStateGpuEField, LqError};

/// `SymplecticEulerRayon` on the device (stateless: every call works on the state it is given).
#[derive(Clone, Copy, Debug, Default, PartialEq, Eq)]
pub struct SymplecticEulerGpu;

type Leap<const D: usize> = SimulationStateLeap<LatticeStateGpuEField<D>, D>;

fn step<const D: usize>(l: &LatticeStateGpuEField<D>, mode: c_int, delta_t: Real) -> Result<LatticeStateGpuEField<D>, LqError> {
    // the reference returns a new state and keeps the old one: a device copy, integrated in place
    let mut out = l.clone();
    check(unsafe { sys::lq_integrate(out.as_raw(), mode, delta_t, 1) })?;
    out.invalidate();
    Ok(out)
}

impl<const D: usize> SymplecticIntegrator<LatticeStateGpuEField<D>, Leap<D>, D> for SymplecticEulerGpu
where
    Direction<D>: DirectionList,
{
    type Error = LqError;

    fn integrate_sync_sync(&self, l: &LatticeStateGpuEField<D>, delta_t: Real) -> Result<LatticeStateGpuEField<D>, LqError> {
        step(l, sys::LQ_SYNC_SYNC, delta_t)
    }

    fn integrate_leap_leap(&self, l: &Leap<D>, delta_t: Real) -> Result<Leap<D>, LqError> {
        Ok(Leap::new_from_state(step(l.state(), sys::LQ_LEAP_LEAP, delta_t)?))
    }

    fn integrate_sync_leap(&self, l: &LatticeStateGpuEField<D>, delta_t: Real) -> Result<Leap<D>, LqError> {
        Ok(Leap::new_from_state(step(l, sys::LQ_SYNC_LEAP, delta_t)?))
    }

    fn integrate_leap_sync(&self, l: &Leap<D>, delta_t: Real) -> Result<LatticeStateGpuEField<D>, LqError> {
        step(l.state(), sys::LQ_LEAP_SYNC, delta_t)
    }

    /// one fused device step (half kick, drift, half kick) instead of sync_leap followed by leap_sync:
    /// the same arithmetic as the trait's default composition
    fn integrate_symplectic(&self, l: &LatticeStateGpuEField<D>, delta_t: Real) -> Result<LatticeStateGpuEField<D>, LqError> {
        step(l, sys::LQ_SYMPLECTIC, delta_t)
    }
}
