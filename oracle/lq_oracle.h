/*
 * lq_oracle.h -- C interface of the CPU oracle for the HMC molecular-dynamics path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++17 restatement of the reference
 * crate lattice-qcd-rs v0.2.1 (Rust) for the hybrid Monte Carlo path.  It is the
 * checker for the CUDA library (tests, the smoke check and the CPU baseline of
 * bench.py) and is never linked into, loaded by or called from the product path.
 *
 * Data layouts are the reference's own (serde of nalgebra/num-complex types):
 *   links  : double[V*D][3 cols][3 rows][re,im]  (column-major 3x3 complex, link = site*D + mu)
 *   efield : double[V][D][8]                     (su(3) coefficients, site-major)
 *   site   : sum_i x_i * L^i, x_0 fastest          (src/lattice.rs:909-916)
 *
 * Every function returns an int status (0 = ok, see OR_* below) unless stated.
 */
#ifndef LQ_ORACLE_H
#define LQ_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    OR_OK = 0,
    OR_ERR_NON_POSITIVE_SIZE = 1, /* LatticeInitializationError::NonPositiveSize */
    OR_ERR_DIM_TOO_SMALL = 2,     /* LatticeInitializationError::DimTooSmall */
    OR_ERR_ZERO_DIMENSION = 3,    /* LatticeInitializationError::ZeroDimension */
    OR_ERR_UNSUPPORTED_D = 4,     /* D outside {2,3,4} */
    OR_ERR_INVALID_NORMAL = 5,    /* StateInitializationError::InvalidParameterNormalDistribution */
    OR_ERR_GAUSS_PROJECTION = 7,  /* StateInitializationError::GaussProjectionError */
    OR_ERR_ZERO_INTEGRATION = 8,  /* MultiIntegrationError::ZeroIntegration */
    OR_ERR_INVALID_ARGUMENT = 9,
    OR_ERR_NOT_CONVERGED = 10     /* projection hit max_steps (the reference loops forever) */
};

/* integrator modes (src/integrator/mod.rs:93-208) */
enum {
    OR_SYNC_SYNC = 0,
    OR_SYNC_LEAP = 1,
    OR_LEAP_LEAP = 2,
    OR_LEAP_SYNC = 3,
    OR_SYMPLECTIC = 4,
    OR_SYMPLECTIC_EXP = 5,            /* symplectic with U' = su3_exp_i(dt sqrt(6)/size E) U */
    OR_SYMPLECTIC_EXP_NORMALIZE = 6   /* the same, then orthonormalize_matrix on every link */
};

/* ---- random numbers: Xoshiro256++ seeded through SplitMix64 ---- */
void *or_rng_new(uint64_t seed);
void or_rng_free(void *rng);
uint64_t or_rng_next_u64(void *rng);
double or_rng_uniform(void *rng, double low, double high);
double or_rng_standard_normal(void *rng);

/* ---- lattice ---- */
int or_lattice_new(int dim, double size, long number_of_points);

/* ---- su(3) algebra (matrices are 18 doubles, column-major complex) ---- */
void or_generators(double *out_8x18);
void or_su3_to_matrix(const double *adj8, double *out18);
void or_su3_exp_i(const double *adj8, double *out18);
void or_su3_exp_r(const double *adj8, double *out18);
void or_orthonormalize(const double *m18, double *out18);
void or_random_su3(void *rng, double *out18);
void or_matmul(const double *a18, const double *b18, double *out18);
void or_determinant(const double *m18, double *out2);

/* ---- field initialisation ---- */
int or_links_random(int dim, int L, void *rng, double *links);
int or_links_cold(int dim, int L, double *links);
int or_efield_normal(int dim, int L, void *rng, double std_dev, double *efield);

/* ---- observables ---- */
int or_hamiltonian_links(int dim, int L, double beta, const double *links, double *out);
int or_hamiltonian_efield(int dim, int L, double beta, const double *efield, double *out);
int or_average_trace_plaquette(int dim, int L, const double *links, double *re, double *im);
/* LinkMatrix::clover / f_mu_nu / magnetic_field (src/field.rs:806-871) at one point */
int or_clover(int dim, int L, const double *links, long site, int i, int i_pos, int j, int j_pos, double *out18);
int or_f_mu_nu(int dim, int L, double size, const double *links, long site, int i, int j, double *out18);
int or_magnetic_field(int dim, int L, double size, const double *links, long site, int k, double *out18);
/* MetropolisHastingsSweep / HeatBathSweep in checkerboard order, Philox stream per link (see the source) */
int or_metropolis_sweep(int dim, int L, double beta, const double *links_in, int n_update, double spread,
                        uint64_t seed, uint64_t sweep, double *links_out, long *n_accepted, double *prob_sum);
int or_heat_bath_sweep(int dim, int L, double beta, const double *links_in, uint64_t seed, uint64_t sweep,
                       double *links_out);
/* OverrelaxationSweepRotation (method 0) / OverrelaxationSweepReverse (1) in checkerboard order, and
 * one link's update from its link and staple matrices (see the source) */
int or_overrelaxation_sweep(int dim, int L, const double *links_in, int method, double *links_out);
int or_overrelax_link(const double *link18, const double *staple18, int method, double *out18);
int or_gauss(int dim, int L, const double *links, const double *efield, long site, double *out18);
int or_gauss_sum_div(int dim, int L, const double *links, const double *efield, double *out);
int or_project_to_gauss(int dim, int L, const double *links, const double *efield_in,
                        double *efield_out, int max_steps, int *steps_done);
int or_normalize(int dim, int L, double *links);

/* derivative_e for every site (force on every link), src/simulation/state.rs:1420-1448 */
int or_derivative_e(int dim, int L, double size, const double *links, double *force);
/* derivative_u for every link, src/simulation/state.rs:1407-1417 */
int or_derivative_u(int dim, int L, double size, const double *links, const double *efield,
                    double *du);

/* ---- integrators (SymplecticEulerRayon), n >= 1 repetitions of `mode` ---- */
int or_integrate(int dim, int L, double size, const double *links_in, const double *efield_in,
                 int mode, double dt, int n, double *links_out, double *efield_out);
/* simulate_using_leapfrog_n: sync->leap, (n-1) leap->leap, leap->sync */
int or_leapfrog_n(int dim, int L, double size, const double *links_in, const double *efield_in,
                  double dt, int n, double *links_out, double *efield_out);

/* ---- one HybridMonteCarloDiagnostic step with injected momenta and uniform ----
 * efield_raw: the N(0, 0.5/beta) draw before the Gauss projection.
 * Accept iff prob >= 1 or uniform < prob (rand 0.8 Bernoulli semantics).
 * links_out receives the new state on accept and a copy of links_in on reject.
 * h_old/h_new: hamiltonian_total of the projected start state and the integrated state. */
int or_hmc_trajectory(int dim, int L, double size, double beta, const double *links_in,
                      const double *efield_raw, double dt, int n_steps, double uniform,
                      int max_gauss_steps, double *links_out, double *efield_out,
                      int *accepted, double *prob, double *h_old, double *h_new,
                      int *gauss_steps);

/* thread control for the CPU baseline (OpenMP) */
void or_set_threads(int n);
int or_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
