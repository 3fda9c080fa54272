/*
 * lqgpu.h -- C ABI of the GB300 (sm_103a) HMC molecular-dynamics library.
 *
 * A device-resident replacement for the hot path of lattice-qcd-rs v0.2.1: the state
 * types LatticeStateDefault<D> / LatticeStateEFSyncDefault<LatticeStateDefault<D>, D>,
 * the SymplecticIntegrator SymplecticEulerRayon, and the per-trajectory work of
 * HybridMonteCarloDiagnostic.  Each entry point names the reference item it replaces
 * (paths relative to the reference crate root).
 *
 * Conventions
 *  - Every function returns an int32 status: LQ_OK (0) or one of the LQ_ERR_* codes.
 *    No C++ exception crosses this boundary; nothing traps on the device.
 *  - A handle is used by one host thread at a time (externally synchronised).
 *  - All device work of a handle runs on the handle's CUDA stream (lq_state_set_stream).
 *    Functions that return host values synchronise that stream.
 *  - Host arrays use the reference's serde layouts:
 *      links  : double[V*D][3 cols][3 rows][2]  column-major 3x3 complex (nalgebra),
 *               link index = site*D + mu  (src/lattice.rs:925-929)
 *      efield : double[V][D][8]           su(3) coefficients e^a of E = e^a T^a
 *               (src/field.rs:1025-1027)
 *      site   : sum_i x_i L^i, x_0 fastest (src/lattice.rs:909-916)
 *  - D must be 2, 3 or 4; any other D returns LQ_ERR_UNSUPPORTED_DIM.
 */
#ifndef LQGPU_H
#define LQGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
enum lq_status {
    LQ_OK = 0,
    /* LatticeInitializationError (src/error.rs:219-241) */
    LQ_ERR_NON_POSITIVE_SIZE = 1,
    LQ_ERR_DIM_TOO_SMALL = 2,
    LQ_ERR_ZERO_DIMENSION = 3,
    LQ_ERR_UNSUPPORTED_DIM = 4,
    /* StateInitializationError (src/error.rs:124-171) */
    LQ_ERR_INVALID_NORMAL = 5,      /* InvalidParameterNormalDistribution: 0.5/beta not a valid std dev */
    LQ_ERR_INCOMPATIBLE_SIZE = 6,   /* IncompatibleSize */
    LQ_ERR_GAUSS_PROJECTION = 7,    /* GaussProjectionError (NaN residual, src/field.rs:1282-1284) */
    /* MultiIntegrationError (src/error.rs:93-118) */
    LQ_ERR_ZERO_INTEGRATION = 8,    /* ZeroIntegration */
    /* library errors without a reference counterpart */
    LQ_ERR_INVALID_ARGUMENT = 9,
    LQ_ERR_NOT_CONVERGED = 10,      /* Gauss projection reached max_steps (the reference loops forever) */
    LQ_ERR_WRONG_STATE_KIND = 11,   /* leap-frog call on a synchronous state or vice versa */
    LQ_ERR_NO_PENDING = 12,         /* lq_hmc_decide without a proposal */
    LQ_ERR_CUDA = 20,               /* a CUDA runtime call failed (lq_last_error_string) */
    LQ_ERR_OUT_OF_MEMORY = 21,
    LQ_ERR_NO_DEVICE = 22
};

/* arithmetic of the state */
enum lq_precision {
    LQ_PRECISION_F64 = 0,   /* FP64 throughout: parity form */
    LQ_PRECISION_MIXED = 1, /* FP32 arithmetic (force, kicks, link update, projection) on links and E-field
                               stored as compensated FP32 pairs (hi + lo, error-free two-sum updates);
                               Hamiltonian, Delta H, plaquette and residual sums in FP64; Delta H from
                               difference kernels; reprojection in FP64 */
    LQ_PRECISION_F32 = 2    /* as MIXED but links and E-field stored as plain FP32 (half the bytes,
                               Delta H error grows with the volume) */
};

/* SymplecticIntegrator methods (src/integrator/mod.rs:93-208) */
enum lq_integration_mode {
    LQ_SYNC_SYNC = 0,   /* integrate_sync_sync:  U += dt dU(E,U);  E += dt F(U)       (both from the old state) */
    LQ_SYNC_LEAP = 1,   /* integrate_sync_leap:  E += dt/2 F(U)                       (state becomes leap-frog) */
    LQ_LEAP_LEAP = 2,   /* integrate_leap_leap:  U += dt dU(E,U);  E += dt F(U')      */
    LQ_LEAP_SYNC = 3,   /* integrate_leap_sync:  U += dt dU(E,U);  E += dt/2 F(U')    (state becomes synchronous) */
    LQ_SYMPLECTIC = 4,  /* integrate_symplectic: E += dt/2 F(U); U += dt dU(E,U); E += dt/2 F(U') */
    /* no counterpart in the reference's integrators: the symplectic step with the link moved on the
     * group, U' = exp(i dt sqrt(2 C_A)/size E) U, the exponential by the Cayley-Hamilton recursion
     * of su3::su3_exp_i (src/su3.rs:832-855); _REUNITARIZE applies normalize_link_matrices
     * (src/su3.rs:290-309) to every link after each step, in the same kernel */
    LQ_SYMPLECTIC_EXP = 5,
    LQ_SYMPLECTIC_EXP_REUNITARIZE = 6
};

/* link update used by lq_hmc_propose / lq_hmc_trajectory (lq_state_set_link_update) */
enum lq_link_update {
    LQ_LINK_UPDATE_EULER = 0,            /* integrate_link, the reference's first-order update (default) */
    LQ_LINK_UPDATE_EXP = 1,              /* exp(i dt c E) U */
    LQ_LINK_UPDATE_EXP_REUNITARIZE = 2   /* exp(i dt c E) U, then orthonormalize_matrix per step */
};

typedef struct lq_state lq_state;

/* ---------------------------------------------------------------- lifetime */

/* LatticeCyclic::new (src/lattice.rs:190-201) + LatticeStateDefault::new_cold
 * (src/simulation/state.rs:670-678) + LatticeStateEFSyncDefault::new_e_cold
 * (src/simulation/state.rs:1111-1120): a state of V = L^dim sites with U = 1, E = 0, t = 0.
 * size: the lattice spacing parameter (forces scale as 1/size); beta: coupling.
 * Validation order and errors follow LatticeCyclic::new, then LQ_ERR_UNSUPPORTED_DIM. */
int lq_state_create(int dim, int L, double size, double beta, int precision, lq_state **out);
int lq_state_destroy(lq_state *s);
/* Clone for State: Clone (src/simulation/monte_carlo/hybrid_monte_carlo.rs:318); same stream. */
int lq_state_clone(const lq_state *s, lq_state **out);
/* Whole-state checkpoint: the serde derives of LatticeStateDefault / LatticeStateEFSyncDefault
 * (src/simulation/state.rs:653-654, :1046-1047) serialise the lattice, beta, the links, the E-field
 * and t.  lq_state_save writes all of it into a host buffer of lq_state_checkpoint_bytes bytes: a
 * 112-byte little-endian header (magic "LQGPUCK1", version, D, L, precision, size, beta, t, the
 * leap-frog flag, the link update and the projection-loop choice), then the device's link and
 * E-field arrays as stored, compensated lo halves included, so lq_state_load gives a state that
 * continues bitwise as the saved one would (the HMC random streams are the caller's seed and
 * counter).  The image is this library's own format; the serde layouts stay available through
 * lq_links_download / lq_efield_download.  Saving with an undecided HMC proposal returns
 * LQ_ERR_INVALID_ARGUMENT; a buffer of the wrong size LQ_ERR_INCOMPATIBLE_SIZE; lq_state_load
 * rejects a buffer without the magic and version with LQ_ERR_INVALID_ARGUMENT.  The loaded state
 * uses the legacy default stream. */
int lq_state_checkpoint_bytes(const lq_state *s, size_t *bytes);
int lq_state_save(lq_state *s, void *buf, size_t n_bytes);
int lq_state_load(const void *buf, size_t n_bytes, lq_state **out);
/* Attach a cudaStream_t (passed as void*); NULL selects the legacy default stream. */
int lq_state_set_stream(lq_state *s, void *cuda_stream);
/* The Gauss projection's sweep loop (EField::project_to_gauss, src/field.rs:1265-1294) runs as
 * one CUDA graph launch whose convergence test is a device kernel driving a conditional while node
 * (enable = 1, the default), or as host-driven launches with one host read of the residual per
 * test (enable = 0).  Both give the same sweeps and the same field.  A driver that cannot build
 * the graph turns it off for the state.  Without a step limit (max_steps <= 0) the graph's device-side loop
 * still stops after 10001 sweeps with LQ_ERR_NOT_CONVERGED, the limit of a batch's loop too. */
int lq_state_set_projection_graph(lq_state *s, int enable);
/* Getters: LatticeCyclic::dim/size, LatticeState::beta, LatticeStateWithEField::t,
 * number_of_points (src/lattice.rs:208-233). is_leap = 1 between sync_leap and leap_sync. */
int lq_state_info(const lq_state *s, int *dim, int *L, double *size, double *beta, int *precision,
                  long long *n_sites, long long *t, int *is_leap);
int lq_state_set_beta(lq_state *s, double beta);
/* choose the link update of the HMC proposal (lq_link_update); Euler, the reference's, by default */
int lq_state_set_link_update(lq_state *s, int link_update);
/* Device bytes held by the state (links buffers, E, Gauss buffer, staging; an FP64 state adds a
 * scratch array of 82 reals per link: its Gauss projection's transport tables and its MD step's
 * force parts). */
int lq_state_device_bytes(const lq_state *s, size_t *bytes);

/* ---------------------------------------------------------------- fields */

/* LatticeState::set_link_matrix / link_matrix (src/simulation/state.rs:73-81, :808-815).
 * n_doubles must be V*D*18, else LQ_ERR_INCOMPATIBLE_SIZE (the reference panics). */
int lq_links_upload(lq_state *s, const double *links, size_t n_doubles);
int lq_links_download(lq_state *s, double *links, size_t n_doubles);
/* LinkMatrix::new_cold (src/field.rs:703-707) */
int lq_links_set_cold(lq_state *s);
/* LinkMatrix::new_determinist with su3::random_su3 (src/field.rs:646-659, src/su3.rs:322-355),
 * drawn on the device from a Philox4x32-10 stream keyed by seed (not the Rust RNG stream). */
int lq_links_random(lq_state *s, uint64_t seed);

/* LatticeStateWithEField::set_e_field / e_field (src/simulation/state.rs:1387-1399).
 * n_doubles must be V*D*8. */
int lq_efield_upload(lq_state *s, const double *efield, size_t n_doubles);
int lq_efield_download(lq_state *s, double *efield, size_t n_doubles);
/* EField::new_cold (src/field.rs:1126-1131) */
int lq_efield_set_cold(lq_state *s);
/* EField::new_determinist with Normal(0, std_dev) (src/field.rs:1086-1099): every coefficient
 * drawn on the device (Philox4x32-10 + Box-Muller) from (seed, counter). */
int lq_efield_random_normal(lq_state *s, uint64_t seed, uint64_t counter, double std_dev);

/* ---------------------------------------------------------------- observables */

/* LatticeState::hamiltonian_links (src/simulation/state.rs:821-849): beta sum_x sum_{mu<nu} (1 - Re Tr P/3) */
int lq_hamiltonian_links(lq_state *s, double *out);
/* LatticeStateWithEField::hamiltonian_efield (src/simulation/state.rs:1370-1385): beta sum e^2/2 */
int lq_hamiltonian_efield(lq_state *s, double *out);
/* LatticeStateWithEField::hamiltonian_total (src/simulation/state.rs:229-231) */
int lq_hamiltonian_total(lq_state *s, double *out);
/* LatticeState::average_trace_plaquette (src/field.rs:775-804): sum Tr P / (V D(D-1)/2) */
int lq_average_trace_plaquette(lq_state *s, double *re, double *im);
/* EField::gauss_sum_div (src/field.rs:1199-1220): sum_x |Tr((sum_a T^a) G(x))| */
int lq_gauss_sum_div(lq_state *s, double *out);
/* EField::gauss at every site (src/field.rs:1174-1195), as 8 coefficients g^a = 2 Re Tr(T^a G(x)),
 * out: double[V][8]. */
int lq_gauss_download(lq_state *s, double *out, size_t n_doubles);

/* ---------------------------------------------------------------- updates */

/* EField::project_to_gauss (src/field.rs:1265-1294): one projection step, then blocks of four
 * until gauss_sum_div <= eps * V * 320 (eps of the state's storage type).  max_steps > 0 caps
 * the steps (LQ_ERR_NOT_CONVERGED); a NaN residual gives LQ_ERR_GAUSS_PROJECTION. */
int lq_project_gauss(lq_state *s, int max_steps, int *steps_done);
/* LatticeStateDefault::normalize_link_matrices (src/simulation/state.rs:754-756):
 * su3::orthonormalize_matrix on every link (src/su3.rs:290-309), computed in FP64. */
int lq_normalize_link_matrices(lq_state *s);

/* SymplecticIntegrator for SymplecticEulerRayon (src/integrator/symplectic_euler_rayon.rs:120-252),
 * repeated n times as simulate_*_n does (src/simulation/state.rs:399-491, :603-647).
 * n == 0 gives LQ_ERR_ZERO_INTEGRATION.  SYNC_LEAP requires a synchronous state and leaves a
 * leap-frog state; LEAP_LEAP requires leap-frog; LEAP_SYNC requires leap-frog and leaves a
 * synchronous state; SYNC_SYNC / SYMPLECTIC require a synchronous state (else
 * LQ_ERR_WRONG_STATE_KIND).  t advances as in the reference (sync_leap does not advance it).
 * LQ_SYMPLECTIC_EXP(_REUNITARIZE) behave as LQ_SYMPLECTIC with the exponential link update. */
int lq_integrate(lq_state *s, int mode, double dt, int n);
/* simulate_using_leapfrog_n (src/simulation/state.rs:318-357) */
int lq_leapfrog_n(lq_state *s, double dt, int n);

/* ---------------------------------------------------------------- local Monte Carlo sweeps
 * MetropolisHastingsSweep::next_element (src/simulation/monte_carlo/metropolis_hastings_sweep.rs:147-177,
 * proposals new = prod_k orthonormalize(random_su3_close_to_unity(spread)) U, accepted with
 * min(1, exp(-Delta S)), Delta S = -Re Tr((U' - U) A) beta / 3 with the staple A of mod.rs:339-362) and
 * HeatBathSweep::next_element (heat_bath.rs:88-121, the pseudo heat bath on the three SU(2)
 * subgroups).  One call is one sweep over every link, in checkerboard order (for each direction,
 * the links on even sites, then on odd sites) instead of the reference's lattice order, so L must be
 * even (else LQ_ERR_INVALID_ARGUMENT).  Random numbers: a Philox4x32-10 stream per link keyed by seed,
 * counter = sweep (not the rand crate's streams).  lq_metropolis_sweep returns the number of accepted
 * updates and the mean acceptance probability (number_replace_last, prob_replace_mean); its argument
 * checks are MetropolisHastingsSweep::new's (n_update >= 1, 0 < spread < 1). */
int lq_metropolis_sweep(lq_state *s, int n_update, double spread, uint64_t seed, uint64_t sweep,
                        long long *n_accepted, double *prob_mean);
int lq_heat_bath_sweep(lq_state *s, uint64_t seed, uint64_t sweep);
/* OverrelaxationSweepRotation (LQ_OVERRELAX_ROTATION) / OverrelaxationSweepReverse
 * (LQ_OVERRELAX_REVERSE), src/simulation/monte_carlo/overrelaxation.rs: every link replaced by
 * rot U^dag rot with rot = U_s V_s^dag, or by U_s reverse(U_s^dag U V_s) V_s^dag, from the singular
 * value decomposition U_s S V_s^dag of the Monte Carlo staple's adjoint (reverse negates the
 * off-diagonal entries); the link Hamiltonian is conserved.  Checkerboard order as the sweeps above
 * (L even), arithmetic in double for every storage form; no random numbers. */
enum { LQ_OVERRELAX_ROTATION = 0, LQ_OVERRELAX_REVERSE = 1 };
int lq_overrelaxation_sweep(lq_state *s, int method);

/* ---------------------------------------------------------------- clover observables
 * LinkMatrix::f_mu_nu and magnetic_field_vec (src/field.rs:822-871) at every site, from the clover
 * C_ij = P_ij + P_{j,-i} + P_{-i,-j} + P_{-j,i} (src/field.rs:806-820):
 *   lq_field_strength: F_ij = (C_ij - C_ji) / (8 size^2) for the planes i < j in the order
 *     (0,1), (0,2), ..., (D-2,D-1); out double[V][D(D-1)/2][18] (3x3 complex, serde layout);
 *     F_ji = -F_ij.
 *   lq_magnetic_field: B_k = sum_{i,j} eps(k,i,j) F_ij / (2i) for k = 0..D-1 with the three-index
 *     levi_civita (src/utils.rs:306-318); out double[V][D][18] (zero for D = 2). */
int lq_field_strength(lq_state *s, double *out, size_t n_doubles);
int lq_magnetic_field(lq_state *s, double *out, size_t n_doubles);

/* ---------------------------------------------------------------- differentiation
 * The gauge force is the adjoint of the Wilson action: a forward / backward pair in the shape of
 * an autograd function.  No reference counterpart as an API; the reference's force is
 * derivative_e (src/simulation/state.rs:1420-1448), which equals -sqrt(2 C_A)/(size beta) times
 * the backward below. */
/* forward: S = beta sum_x sum_{mu<nu} (1 - Re Tr P / 3), the same value as lq_hamiltonian_links */
int lq_wilson_action(lq_state *s, double *out);
/* backward: dS/dtheta^a for U_mu(x) -> exp(i theta^a T^a) U_mu(x), every link,
 * out: double[V][D][8] (the E-field layout) = beta/3 Im Tr(T^a U_mu(x) Sigma_mu(x)) */
int lq_wilson_action_backward(lq_state *s, double *grad, size_t n_doubles);
/* U_link <- exp(i angle T^a) U_link for one link (link = site*D + mu, a = generator 0..7), for
 * finite-difference probes of the action */
int lq_link_rotate(lq_state *s, long long link, int generator, double angle);

/* Reverse-mode adjoint of a leap-frog trajectory.  No counterpart in the reference.
 * Runs n_steps symplectic steps (LQ_SYMPLECTIC with the reference's first-order link update,
 * the HMC proposal's integrator) from the state's links U0 and momenta E0 -- the state itself
 * is left unchanged -- and differentiates
 *   objective O = Re average_trace_plaquette(U_n) / 3
 * backwards through every kick and drift: grad_links = dO/dU0 as a complex cotangent per
 * link (dO/dRe U + i dO/dIm U, serde link layout), grad_efield = dO/dE0 (E-field layout), and
 *   d_objective_d_beta = dO/dbeta for momenta drawn by scaling one fixed normal field,
 *   E0(beta) = E0 beta0 / beta (the standard deviation is 0.5/beta); the molecular dynamics
 *   itself does not depend on beta (the reference's force has no beta factor).
 * Memory: checkpoints of the state entering every c-th step (c = checkpoint_every, 0: the
 * default ceil(sqrt(n_steps))), each segment recomputed once in the reverse pass; work_bytes
 * returns the device bytes of this work (allocated for the call and freed before it returns).
 * The FP32 forms run the adjoint in FP32 on the hi parts of the links and momenta.
 * Outputs may be NULL; n_*_doubles as lq_links_download / lq_efield_download. */
int lq_leapfrog_adjoint(lq_state *s, double dt, int n_steps, int checkpoint_every, double *objective,
                        double *d_objective_d_beta, double *grad_links, size_t n_link_doubles, double *grad_efield,
                        size_t n_efield_doubles, size_t *work_bytes);

/* ---------------------------------------------------------------- HMC
 * HybridMonteCarloDiagnostic::next_element (src/simulation/monte_carlo/hybrid_monte_carlo.rs:465-471,
 * :573-613), split as the reference splits it:
 *   refresh     : new_random_e_state (src/simulation/state.rs:1093-1108) -- draw E ~ N(0, 0.5/beta)
 *                 then project_to_gauss; lq_hmc_refresh draws on the device, lq_hmc_refresh_upload
 *                 takes the drawn field from the host (test mode).  The projection works on the
 *                 hi parts of a compensated (mixed) field and clears the lo parts when it
 *                 finishes, so the field enters with lo = 0 (after a failed projection the
 *                 field is its hi parts).
 *   propose     : simulate_symplectic_n_auto(dt, n) + probability_of_replacement
 *                 prob = clamp(exp(H_old - H_new), 0, 1); the start state is kept.
 *   decide      : Bernoulli(prob) -- accept = 1 keeps the proposal, 0 restores the start state
 *                 (LatticeStateDefault only: the E-field is dropped by state_owned).
 *   trajectory  : all four with accept = (prob >= 1 || uniform < prob), the rand 0.8 Bernoulli rule. */
int lq_hmc_refresh(lq_state *s, uint64_t seed, uint64_t counter, int max_gauss_steps, int *gauss_steps);
int lq_hmc_refresh_upload(lq_state *s, const double *efield_raw, size_t n_doubles, int max_gauss_steps,
                          int *gauss_steps);
/* Pipelined test mode (no counterpart in the reference): lq_efield_prefetch starts the host -> device
 * copy of the next trajectory's drawn momenta on a copy stream of the state and returns at once;
 * lq_hmc_refresh_prefetched then does what lq_hmc_refresh_upload does with them.  Overlapping the
 * copy of trajectory k+1 with the work of trajectory k hides it.  The host buffer must stay valid and
 * unchanged until the lq_hmc_refresh_prefetched that consumes it returns; page-locked (pinned) host
 * memory makes the copy asynchronous.  lq_hmc_refresh_prefetched without a prefetch returns
 * LQ_ERR_NO_PENDING. */
int lq_efield_prefetch(lq_state *s, const double *efield_raw, size_t n_doubles);
int lq_hmc_refresh_prefetched(lq_state *s, int max_gauss_steps, int *gauss_steps);
int lq_hmc_propose(lq_state *s, double dt, int n_steps, double *prob, double *h_old, double *h_new);
int lq_hmc_decide(lq_state *s, int accept);
int lq_hmc_trajectory(lq_state *s, double dt, int n_steps, uint64_t seed, uint64_t counter, double uniform,
                      int max_gauss_steps, int *accepted, double *prob, double *delta_h, int *gauss_steps);

/* ---------------------------------------------------------------- profiling
 * Per-kernel-class launch counters timed with CUDA events on the state's stream (no
 * reference counterpart: the reference has no tracing).  While enabled, every launch of
 * the state is bracketed by an event pair; totals accumulate at each synchronisation. */
enum lq_kernel_class {
    LQ_KERNEL_MD = 0,         /* the MD step: fused force/kick/drift (k_md_site; FP64 k_md_plaq + k_md_update) */
    LQ_KERNEL_GAUSS = 1,       /* Gauss law G(x) + residual partials (k_gauss; FP64 projection k_gauss_adj) */
    LQ_KERNEL_GAUSS_SWEEP = 2, /* projection sweep (k_gauss_sweep; FP64 k_gauss_step_adj; a projection graph) */
    LQ_KERNEL_PLAQUETTE = 3,  /* plaquette / hamiltonian_links partials (k_plaquette) */
    LQ_KERNEL_REDUCE = 4,     /* sum of squares and final reductions */
    LQ_KERNEL_OTHER = 5,      /* layout conversion, initialisation, reprojection */
    LQ_KERNEL_CLASSES = 6
};
int lq_profile_enable(lq_state *s, int on);
/* Index checks, no reference counterpart (a stand-in for a memory checker): in a library built with
 * -DLQ_BOUNDS_CHECK=1 the kernels compare every site
 * index they form (neighbours, coordinates) and every tile plane with its bound, count a bad one
 * instead of using it (the access goes to index 0) and keep the first.  *enabled: 1 in such a build,
 * 0 otherwise (then *violations is 0 and no device call is made).  *first_bad: the first bad index
 * + 1 (0: none); a plane index reads (planes << 32) | plane.  reset != 0 clears the counters. */
int lq_bounds_check(int *enabled, unsigned long long *violations, unsigned long long *first_bad, int reset);
/* Restrict the profile to the classes whose bit is set in mask (bit k: class k; all by default):
 * launches of the other classes run without events, so timing one class costs the others nothing. */
int lq_profile_classes(lq_state *s, unsigned mask);
/* Measured multiply-add peak of the current device (no reference counterpart): long chains of
 * independent multiply-adds in LQ_PRECISION_F64 or LQ_PRECISION_F32 on every SM, timed with CUDA
 * events at the clocks the device runs at; *flops_per_s counts 2 FLOP per multiply-add.  The
 * denominator of the compute roofline of the FP64 form, whose kernels the FP64 pipe bounds. */
int lq_fma_peak(int precision, double *flops_per_s);
/* launches and total milliseconds of one class since the last reset; also resets when reset != 0 */
int lq_profile_read(lq_state *s, int kernel_class, long long *launches, double *total_ms, int reset);

/* ---------------------------------------------------------------- without allocation
 * No counterpart in the reference.  For callers that cannot let this library allocate device
 * memory: a runtime whose device memory belongs to one pool or arena it manages itself (an
 * embedding framework, a memory-capped MPS client), or a loop that cannot afford the device-wide
 * synchronisation of cudaMalloc / cudaFree.  Computes the plaquette sums of links the caller holds
 * on the device in the serde layout (double[L^dim * dim][18]) and writes them to d_out[0..2] on the
 * device:
 *   d_out[0] = sum (1 - Re Tr P / 3)   (hamiltonian_links = beta * d_out[0])
 *   d_out[1] = sum Re Tr P, d_out[2] = sum Im Tr P
 *              (average_trace_plaquette = (d_out[1] + i d_out[2]) / (L^dim * dim (dim-1) / 2)).
 * The work is enqueued on `stream` (a cudaStream_t; NULL = legacy default stream) and the call
 * returns without synchronising.  Limit: L^dim <= 8,388,608 sites; a larger lattice returns
 * LQ_ERR_INVALID_ARGUMENT with the reason in lq_last_error_string.  Its scratch is one fixed
 * 1.5 MiB device array that every device loading the library holds until the process exits;
 * all calls share it, so calls whose work overlaps on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  The first call on a device looks up the
 * array's device address with that device current and keeps it for the process; make that first
 * call before any stream capture, and do not use the entry point across a device reset
 * (cudaDeviceReset), after which the kept address is stale. */
int lq_plaquette_sums_noalloc(int dim, int L, const double *d_links, double *d_out, void *stream);

/* ---------------------------------------------------------------- batched ensembles
 * The reference's parameter-scan use: many independent HybridMonteCarloDiagnostic runs
 * (src/simulation/monte_carlo/hybrid_monte_carlo.rs:465-471, :573-613), one
 * LatticeStateDefault<D> each (src/simulation/state.rs:577-641), of uneven side length and
 * beta.  The reference runs them one after another; here every ensemble of a batch lives in
 * one set of device arrays and each kernel of a trajectory covers all of them (a per-ensemble
 * offset table), so small lattices do not leave the GPU idle.  An ensemble's trajectory is the
 * same arithmetic as lq_hmc_trajectory of a state of the same precision, with
 *   momenta      : lq_hmc_refresh's device draw, seed = batch seed + ensemble index, counter =
 *                  the ensemble's trajectory counter (lq_batch_set_seed sets both)
 *   accept test  : uniform = the 53-bit Philox value of counter block (0xFFFFFFFF, counter lo,
 *                  counter hi, 4) under the ensemble's key, recorded in the results
 *   Delta H      : -beta/3 sum Re Tr[P' - P] + beta/2 sum (e'^2 - e^2) from difference kernels,
 *                  for every precision (lq_hmc_propose subtracts two Hamiltonians for FP64)
 *   projection   : fused sweeps for every precision (the FP64 state uses two kernels per step),
 *                  per ensemble until its own residual test passes; max_gauss_steps <= 0 means
 *                  10001 (the device loop needs a bound).
 * Ensembles whose projection fails (NaN: LQ_ERR_GAUSS_PROJECTION, or the step limit:
 * LQ_ERR_NOT_CONVERGED) keep their links for that trajectory; the status is in the results. */
typedef struct lq_batch lq_batch;
enum lq_batch_flags {
    LQ_BATCH_USE_GRAPH = 1,         /* replay one captured CUDA graph per trajectory */
    LQ_BATCH_MEASURE_PLAQUETTE = 2  /* record average_trace_plaquette of every ensemble after each trajectory */
};
/* kernel classes of lq_batch_tuning */
enum lq_batch_kernel_class {
    LQ_BATCH_KERNEL_MD = 0,
    LQ_BATCH_KERNEL_SWEEP = 1,
    LQ_BATCH_KERNEL_GAUSS = 2,
    LQ_BATCH_KERNEL_PLAQUETTE_DELTA = 3,
    LQ_BATCH_KERNEL_SUMSQ_DELTA = 4,
    LQ_BATCH_KERNEL_NORMAL = 5,
    LQ_BATCH_KERNEL_PLAQUETTE = 6,
    LQ_BATCH_KERNEL_CLASSES = 7
};
/* n ensembles of dimension dim: ensemble e has L[e] points per direction, lattice size size[e]
 * and beta[e]; cold links.  Errors as lq_state_create, checked per ensemble. */
int lq_batch_create(int dim, int n_ensembles, const int *L, const double *size, const double *beta, int precision,
                    lq_batch **out);
int lq_batch_destroy(lq_batch *b);
int lq_batch_set_stream(lq_batch *b, void *stream);
int lq_batch_info(const lq_batch *b, int *dim, int *n_ensembles, long long *total_links, size_t *device_bytes);
int lq_batch_set_link_update(lq_batch *b, int link_update);
/* Philox keys seed + e and trajectory counters of every ensemble */
int lq_batch_set_seed(lq_batch *b, uint64_t seed, uint64_t counter);
/* ensemble e <- lq_links_random(seed + e) */
int lq_batch_links_random(lq_batch *b, uint64_t seed);
/* one ensemble's links in the serde layout, n = L[e]^dim * dim * 18 doubles */
int lq_batch_links_upload(lq_batch *b, int ensemble, const double *links, size_t n_doubles);
int lq_batch_links_download(lq_batch *b, int ensemble, double *links, size_t n_doubles);
int lq_batch_normalize_link_matrices(lq_batch *b);
/* average_trace_plaquette of every ensemble: re[e], im[e] */
int lq_batch_average_trace_plaquette(lq_batch *b, double *re, double *im);
/* Times each kernel class under candidate launch shapes (one block per work item, or 1, 2, 4, 8
 * waves of resident blocks; directions-fastest or chunks-fastest work order) on the batch's
 * own data and keeps the fastest.  The links are not changed; results of later trajectories do
 * not depend on the shapes. */
int lq_batch_autotune(lq_batch *b, double dt, int reps);
int lq_batch_tuning(const lq_batch *b, int kernel_class, int *grid, int *order, double *ms);
/* n_trajectories HMC trajectories (n_steps leap-frog steps of dt) of every ensemble; results
 * rows 0..n_trajectories-1 of this run. */
int lq_batch_hmc_run(lq_batch *b, double dt, int n_steps, int n_trajectories, int max_gauss_steps, int flags);
/* rows first..first+count-1 of the last run, each array (optional) count * n_ensembles,
 * row-major: delta_h, prob, uniform, accepted, gauss_steps, status, plaquette (<Re Tr P> after
 * the trajectory, with LQ_BATCH_MEASURE_PLAQUETTE) */
int lq_batch_hmc_results(lq_batch *b, int first, int count, double *delta_h, double *prob, double *uniform,
                         int *accepted, int *gauss_steps, int *status, double *plaquette);
/* graph launches since creation */
int lq_batch_graph_launches(const lq_batch *b, long long *launches);
/* Kernel time of eagerly launched trajectories (no reference counterpart): while enabled, every
 * launch of an lq_batch_hmc_run without LQ_BATCH_USE_GRAPH is bracketed by a CUDA event pair on the
 * batch's stream; lq_batch_profile_read returns the launches and their summed milliseconds since
 * the last reset.  Launches inside the captured graph are never bracketed: comparing this sum with
 * the graph's own time on the same trajectories measures the graph's gaps between nodes. */
int lq_batch_profile_enable(lq_batch *b, int on);
int lq_batch_profile_read(lq_batch *b, long long *launches, double *kernel_ms, int reset);

/* ---------------------------------------------------------------- diagnostics */
const char *lq_status_string(int status);
/* Text of the last error on this host thread (CUDA error name and call site). */
const char *lq_last_error_string(void);
/* Library version (major*10000 + minor*100 + patch). */
int lq_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LQGPU_H */
