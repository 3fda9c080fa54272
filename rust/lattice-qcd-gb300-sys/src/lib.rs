//! Raw bindings of liblqgpu (`include/lqgpu.h`): every entry point of the C ABI with the same
//! arguments, and the header's constants.  Each function returns an `lq_status` code (`LQ_OK` = 0);
//! the safe wrappers of the `lattice-qcd-gb300` crate turn them into the reference's types and errors.
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_double, c_int, c_longlong, c_uint, c_ulonglong, c_void};

/// Device-resident HMC state (opaque)
#[repr(C)]
pub struct lq_state {
    _private: [u8; 0],
}
/// Batch of independent ensembles (opaque)
#[repr(C)]
pub struct lq_batch {
    _private: [u8; 0],
}

// lq_status
pub const LQ_OK: c_int = 0;
pub const LQ_ERR_NON_POSITIVE_SIZE: c_int = 1;
pub const LQ_ERR_DIM_TOO_SMALL: c_int = 2;
pub const LQ_ERR_ZERO_DIMENSION: c_int = 3;
pub const LQ_ERR_UNSUPPORTED_DIM: c_int = 4;
pub const LQ_ERR_INVALID_NORMAL: c_int = 5;
pub const LQ_ERR_INCOMPATIBLE_SIZE: c_int = 6;
pub const LQ_ERR_GAUSS_PROJECTION: c_int = 7;
pub const LQ_ERR_ZERO_INTEGRATION: c_int = 8;
pub const LQ_ERR_INVALID_ARGUMENT: c_int = 9;
pub const LQ_ERR_NOT_CONVERGED: c_int = 10;
pub const LQ_ERR_WRONG_STATE_KIND: c_int = 11;
pub const LQ_ERR_NO_PENDING: c_int = 12;
pub const LQ_ERR_CUDA: c_int = 20;
pub const LQ_ERR_OUT_OF_MEMORY: c_int = 21;
pub const LQ_ERR_NO_DEVICE: c_int = 22;

// lq_precision
pub const LQ_PRECISION_F64: c_int = 0;
pub const LQ_PRECISION_MIXED: c_int = 1;
pub const LQ_PRECISION_F32: c_int = 2;

// lq_integration_mode
pub const LQ_SYNC_SYNC: c_int = 0;
pub const LQ_SYNC_LEAP: c_int = 1;
pub const LQ_LEAP_LEAP: c_int = 2;
pub const LQ_LEAP_SYNC: c_int = 3;
pub const LQ_SYMPLECTIC: c_int = 4;
pub const LQ_SYMPLECTIC_EXP: c_int = 5;
pub const LQ_SYMPLECTIC_EXP_REUNITARIZE: c_int = 6;

// lq_link_update
pub const LQ_LINK_UPDATE_EULER: c_int = 0;
pub const LQ_LINK_UPDATE_EXP: c_int = 1;
pub const LQ_LINK_UPDATE_EXP_REUNITARIZE: c_int = 2;

// overrelaxation methods
pub const LQ_OVERRELAX_ROTATION: c_int = 0;
pub const LQ_OVERRELAX_REVERSE: c_int = 1;

// lq_kernel_class
pub const LQ_KERNEL_MD: c_int = 0;
pub const LQ_KERNEL_GAUSS: c_int = 1;
pub const LQ_KERNEL_GAUSS_SWEEP: c_int = 2;
pub const LQ_KERNEL_PLAQUETTE: c_int = 3;
pub const LQ_KERNEL_REDUCE: c_int = 4;
pub const LQ_KERNEL_OTHER: c_int = 5;
pub const LQ_KERNEL_CLASSES: c_int = 6;

// lq_batch_flags
pub const LQ_BATCH_USE_GRAPH: c_int = 1;
pub const LQ_BATCH_MEASURE_PLAQUETTE: c_int = 2;

// lq_batch_kernel_class
pub const LQ_BATCH_KERNEL_MD: c_int = 0;
pub const LQ_BATCH_KERNEL_SWEEP: c_int = 1;
pub const LQ_BATCH_KERNEL_GAUSS: c_int = 2;
pub const LQ_BATCH_KERNEL_PLAQUETTE_DELTA: c_int = 3;
pub const LQ_BATCH_KERNEL_SUMSQ_DELTA: c_int = 4;
pub const LQ_BATCH_KERNEL_NORMAL: c_int = 5;
pub const LQ_BATCH_KERNEL_PLAQUETTE: c_int = 6;
pub const LQ_BATCH_KERNEL_CLASSES: c_int = 7;

extern "C" {
    pub fn lq_state_create(dim: c_int, l: c_int, size: c_double, beta: c_double, precision: c_int, out: *mut *mut lq_state) -> c_int;
    pub fn lq_state_destroy(s: *mut lq_state) -> c_int;
    pub fn lq_state_clone(s: *const lq_state, out: *mut *mut lq_state) -> c_int;
    pub fn lq_state_checkpoint_bytes(s: *const lq_state, bytes: *mut usize) -> c_int;
    pub fn lq_state_save(s: *mut lq_state, buf: *mut c_void, n_bytes: usize) -> c_int;
    pub fn lq_state_load(buf: *const c_void, n_bytes: usize, out: *mut *mut lq_state) -> c_int;
    pub fn lq_state_set_stream(s: *mut lq_state, cuda_stream: *mut c_void) -> c_int;
    pub fn lq_state_set_projection_graph(s: *mut lq_state, enable: c_int) -> c_int;
    pub fn lq_state_info(s: *const lq_state, dim: *mut c_int, l: *mut c_int, size: *mut c_double, beta: *mut c_double, precision: *mut c_int, n_sites: *mut c_longlong, t: *mut c_longlong, is_leap: *mut c_int) -> c_int;
    pub fn lq_state_set_beta(s: *mut lq_state, beta: c_double) -> c_int;
    pub fn lq_state_set_link_update(s: *mut lq_state, link_update: c_int) -> c_int;
    pub fn lq_state_device_bytes(s: *const lq_state, bytes: *mut usize) -> c_int;
    pub fn lq_links_upload(s: *mut lq_state, links: *const c_double, n_doubles: usize) -> c_int;
    pub fn lq_links_download(s: *mut lq_state, links: *mut c_double, n_doubles: usize) -> c_int;
    pub fn lq_links_set_cold(s: *mut lq_state) -> c_int;
    pub fn lq_links_random(s: *mut lq_state, seed: u64) -> c_int;
    pub fn lq_efield_upload(s: *mut lq_state, efield: *const c_double, n_doubles: usize) -> c_int;
    pub fn lq_efield_download(s: *mut lq_state, efield: *mut c_double, n_doubles: usize) -> c_int;
    pub fn lq_efield_set_cold(s: *mut lq_state) -> c_int;
    pub fn lq_efield_random_normal(s: *mut lq_state, seed: u64, counter: u64, std_dev: c_double) -> c_int;
    pub fn lq_hamiltonian_links(s: *mut lq_state, out: *mut c_double) -> c_int;
    pub fn lq_hamiltonian_efield(s: *mut lq_state, out: *mut c_double) -> c_int;
    pub fn lq_hamiltonian_total(s: *mut lq_state, out: *mut c_double) -> c_int;
    pub fn lq_average_trace_plaquette(s: *mut lq_state, re: *mut c_double, im: *mut c_double) -> c_int;
    pub fn lq_gauss_sum_div(s: *mut lq_state, out: *mut c_double) -> c_int;
    pub fn lq_gauss_download(s: *mut lq_state, out: *mut c_double, n_doubles: usize) -> c_int;
    pub fn lq_project_gauss(s: *mut lq_state, max_steps: c_int, steps_done: *mut c_int) -> c_int;
    pub fn lq_normalize_link_matrices(s: *mut lq_state) -> c_int;
    pub fn lq_integrate(s: *mut lq_state, mode: c_int, dt: c_double, n: c_int) -> c_int;
    pub fn lq_leapfrog_n(s: *mut lq_state, dt: c_double, n: c_int) -> c_int;
    pub fn lq_metropolis_sweep(s: *mut lq_state, n_update: c_int, spread: c_double, seed: u64, sweep: u64, n_accepted: *mut c_longlong, prob_mean: *mut c_double) -> c_int;
    pub fn lq_heat_bath_sweep(s: *mut lq_state, seed: u64, sweep: u64) -> c_int;
    pub fn lq_overrelaxation_sweep(s: *mut lq_state, method: c_int) -> c_int;
    pub fn lq_field_strength(s: *mut lq_state, out: *mut c_double, n_doubles: usize) -> c_int;
    pub fn lq_magnetic_field(s: *mut lq_state, out: *mut c_double, n_doubles: usize) -> c_int;
    pub fn lq_wilson_action(s: *mut lq_state, out: *mut c_double) -> c_int;
    pub fn lq_wilson_action_backward(s: *mut lq_state, grad: *mut c_double, n_doubles: usize) -> c_int;
    pub fn lq_link_rotate(s: *mut lq_state, link: c_longlong, generator: c_int, angle: c_double) -> c_int;
    pub fn lq_leapfrog_adjoint(s: *mut lq_state, dt: c_double, n_steps: c_int, checkpoint_every: c_int, objective: *mut c_double, d_objective_d_beta: *mut c_double, grad_links: *mut c_double, n_link_doubles: usize, grad_efield: *mut c_double, n_efield_doubles: usize, work_bytes: *mut usize) -> c_int;
    pub fn lq_hmc_refresh(s: *mut lq_state, seed: u64, counter: u64, max_gauss_steps: c_int, gauss_steps: *mut c_int) -> c_int;
    pub fn lq_hmc_refresh_upload(s: *mut lq_state, efield_raw: *const c_double, n_doubles: usize, max_gauss_steps: c_int, gauss_steps: *mut c_int) -> c_int;
    pub fn lq_efield_prefetch(s: *mut lq_state, efield_raw: *const c_double, n_doubles: usize) -> c_int;
    pub fn lq_hmc_refresh_prefetched(s: *mut lq_state, max_gauss_steps: c_int, gauss_steps: *mut c_int) -> c_int;
    pub fn lq_hmc_propose(s: *mut lq_state, dt: c_double, n_steps: c_int, prob: *mut c_double, h_old: *mut c_double, h_new: *mut c_double) -> c_int;
    pub fn lq_hmc_decide(s: *mut lq_state, accept: c_int) -> c_int;
    pub fn lq_hmc_trajectory(s: *mut lq_state, dt: c_double, n_steps: c_int, seed: u64, counter: u64, uniform: c_double, max_gauss_steps: c_int, accepted: *mut c_int, prob: *mut c_double, delta_h: *mut c_double, gauss_steps: *mut c_int) -> c_int;
    pub fn lq_profile_enable(s: *mut lq_state, on: c_int) -> c_int;
    pub fn lq_bounds_check(enabled: *mut c_int, violations: *mut c_ulonglong, first_bad: *mut c_ulonglong, reset: c_int) -> c_int;
    pub fn lq_profile_classes(s: *mut lq_state, mask: c_uint) -> c_int;
    pub fn lq_fma_peak(precision: c_int, flops_per_s: *mut c_double) -> c_int;
    pub fn lq_profile_read(s: *mut lq_state, kernel_class: c_int, launches: *mut c_longlong, total_ms: *mut c_double, reset: c_int) -> c_int;
    pub fn lq_plaquette_sums_noalloc(dim: c_int, l: c_int, d_links: *const c_double, d_out: *mut c_double, stream: *mut c_void) -> c_int;
    pub fn lq_batch_create(dim: c_int, n_ensembles: c_int, l: *const c_int, size: *const c_double, beta: *const c_double, precision: c_int, out: *mut *mut lq_batch) -> c_int;
    pub fn lq_batch_destroy(b: *mut lq_batch) -> c_int;
    pub fn lq_batch_set_stream(b: *mut lq_batch, stream: *mut c_void) -> c_int;
    pub fn lq_batch_info(b: *const lq_batch, dim: *mut c_int, n_ensembles: *mut c_int, total_links: *mut c_longlong, device_bytes: *mut usize) -> c_int;
    pub fn lq_batch_set_link_update(b: *mut lq_batch, link_update: c_int) -> c_int;
    pub fn lq_batch_set_seed(b: *mut lq_batch, seed: u64, counter: u64) -> c_int;
    pub fn lq_batch_links_random(b: *mut lq_batch, seed: u64) -> c_int;
    pub fn lq_batch_links_upload(b: *mut lq_batch, ensemble: c_int, links: *const c_double, n_doubles: usize) -> c_int;
    pub fn lq_batch_links_download(b: *mut lq_batch, ensemble: c_int, links: *mut c_double, n_doubles: usize) -> c_int;
    pub fn lq_batch_normalize_link_matrices(b: *mut lq_batch) -> c_int;
    pub fn lq_batch_average_trace_plaquette(b: *mut lq_batch, re: *mut c_double, im: *mut c_double) -> c_int;
    pub fn lq_batch_autotune(b: *mut lq_batch, dt: c_double, reps: c_int) -> c_int;
    pub fn lq_batch_tuning(b: *const lq_batch, kernel_class: c_int, grid: *mut c_int, order: *mut c_int, ms: *mut c_double) -> c_int;
    pub fn lq_batch_hmc_run(b: *mut lq_batch, dt: c_double, n_steps: c_int, n_trajectories: c_int, max_gauss_steps: c_int, flags: c_int) -> c_int;
    pub fn lq_batch_hmc_results(b: *mut lq_batch, first: c_int, count: c_int, delta_h: *mut c_double, prob: *mut c_double, uniform: *mut c_double, accepted: *mut c_int, gauss_steps: *mut c_int, status: *mut c_int, plaquette: *mut c_double) -> c_int;
    pub fn lq_batch_graph_launches(b: *const lq_batch, launches: *mut c_longlong) -> c_int;
    pub fn lq_batch_profile_enable(b: *mut lq_batch, on: c_int) -> c_int;
    pub fn lq_batch_profile_read(b: *mut lq_batch, launches: *mut c_longlong, kernel_ms: *mut c_double, reset: c_int) -> c_int;
    pub fn lq_status_string(status: c_int) -> *const c_char;
    pub fn lq_last_error_string() -> *const c_char;
    pub fn lq_version() -> c_int;
}
