// state.hpp -- the device-resident HMC state behind the lq_state handle, and the
// per-(D, precision) table of device operations.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "block_order.hpp"
#include "lqgpu.h"

namespace lq {

struct Ops;

// CUDA-event launch counters (lq_profile_enable / lq_profile_read)
constexpr int kProfPool = 1024;
constexpr int kProfClasses = 6;
struct Prof {
    cudaEvent_t ev[2 * kProfPool];
    int cls[kProfPool];
    int cnt[kProfPool]; // kernels a slot covers (1 for a launch, more for a graph)
    int n = 0;
    long long launches[kProfClasses] = {0, 0, 0, 0, 0, 0};
    double ms[kProfClasses] = {0, 0, 0, 0, 0, 0};
};

// Buffers are untyped here; the element type is double or float according to `precision`.
struct State {
    int dim = 0;
    int L = 0;
    uint32_t V = 0;
    double size = 1.0;
    double beta = 1.0;
    int precision = LQ_PRECISION_F64;
    size_t real_bytes = 8; // sizeof(T)
    int comp = 0;          // 1: compensated (hi, lo) storage of links and E-field
    cudaStream_t stream = nullptr;

    void *U[3] = {nullptr, nullptr, nullptr}; // link buffers (SoA); U[cur] is the state
    int cur = 0;
    void *E = nullptr;     // E-field (SoA)
    void *E_alt = nullptr; // second E buffer (projection sweeps are double-buffered)
    void *G = nullptr;     // Gauss law G(x): Hermitian matrix, 9 reals per site (FP64 projection: components)
    void *G_alt = nullptr;
    // FP64 scratch, 82 reals per link: the Gauss projection's transport tables of the links it
    // projects on, and between projections the MD step's force parts (D x 8 reals per link)
    void *R = nullptr;
    double *partial = nullptr;
    uint32_t partial_slots = 0; // slots per row of `partial`
    double *d_out = nullptr;    // device scalars
    double *h_out = nullptr;    // pinned host mirror of d_out
    void *staging = nullptr;    // f64 AoS staging for uploads/downloads
    size_t staging_bytes = 0;
    // momenta prefetch (lq_efield_prefetch): a second staging buffer filled on its own stream
    void *prefetch = nullptr;
    size_t prefetch_bytes = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t prefetch_done = nullptr; // the copy has landed
    cudaEvent_t prefetch_free = nullptr; // the last prefetched field has been consumed
    int prefetch_pending = 0;

    // the Gauss projection's sweep loop as a CUDA graph whose while node the device-side check
    // drives (lq_state_set_projection_graph): one instantiation per (link buffer, E buffer order,
    // G buffer order, step limit) met, built on first use; 12 entries hold every combination of the
    // 3 link buffers and 2 x 2 buffer orders (an HMC loop meets 6; the FP64 form, whose sweeps work in
    // place, 3)
    struct ProjGraph {
        const void *U;
        const void *E;
        const void *G;
        int max_steps;
        cudaGraphExec_t exec;
    };
    static constexpr int kProjGraphs = 12;
    int proj_graph = 1;
    ProjGraph proj[kProjGraphs] = {};
    int n_proj = 0;
    int *d_proj = nullptr; // device: sweeps done, status
    cudaStream_t cap_main = nullptr, cap_body = nullptr;

    long long t = 0;
    int leap = 0;
    int link_update = LQ_LINK_UPDATE_EULER; // of the HMC proposal

    // HMC proposal bookkeeping
    int has_pending = 0;
    int pending_buf = -1;
    double pending_hu_old = 0.0, pending_hu_new = 0.0, pending_dh = 0.0;
    // cached hamiltonian_links of U[cur] (reductions are deterministic, so the cached value
    // equals a recomputation)
    int hu_valid = 0;
    double hu = 0.0;

    const Ops *ops = nullptr;
    Prof *prof = nullptr;       // non-null while profiling is enabled
    unsigned prof_mask = ~0u;   // the kernel classes the profile times (lq_profile_classes)
    // launch order of the per-site stencil kernels' blocks (block_order.hpp)
    BlockOrder block_order = {0, 1, 1, 1};

    // arrays are stored in tiles of 32 sites (padded; see tix() in su3.cuh)
    size_t padded_sites() const { return ((size_t)V + 31) / 32 * 32; }
    size_t link_elems() const { return padded_sites() * dim * 9; }   // complex elements
    size_t link_bytes() const { return link_elems() * 2 * real_bytes * (comp ? 2 : 1); }
    size_t efield_elems() const { return padded_sites() * dim * 8; } // reals (hi part)
    size_t efield_bytes() const { return efield_elems() * real_bytes * (comp ? 2 : 1); }
    // G: 9 reals per site in the Hermitian form, 10 (9 components and a pad) in the FP64 projection's
    size_t gauss_bytes() const { return padded_sites() * (precision == LQ_PRECISION_F64 ? 10 : 9) * real_bytes; }
    size_t adjoint_bytes() const { return padded_sites() * dim * 82 * real_bytes; }
};

// Device operations of one (D, T, COMP) instantiation.  Launches are asynchronous on
// s.stream and return cudaError_t of the launch.
struct Ops {
    cudaError_t (*links_from_aos)(State &s, const double *d_aos, void *dst);
    cudaError_t (*links_to_aos)(State &s, const void *src, double *d_aos);
    cudaError_t (*links_cold)(State &s, void *dst);
    cudaError_t (*links_random)(State &s, void *dst, uint64_t seed);
    cudaError_t (*efield_from_aos)(State &s, const double *d_aos);
    cudaError_t (*efield_to_aos)(State &s, const void *E, double *d_aos);
    cudaError_t (*efield_normal)(State &s, uint64_t seed, uint64_t counter, double sd);
    // md: mode bits MD_KICK | MD_DRIFT | MD_DRIFT_OLD_E; h1, h2 kick step sizes; dt drift step;
    // E is read from Ein and written to Eout (equal for an in-place update)
    cudaError_t (*md)(State &s, const void *Uin, void *Uout, const void *Ein, void *Eout, int mode, double h1,
                      double h2, double dt);
    // gauss: G <- gauss(E, U), residual partials into s.partial (row 0), returns #partials
    cudaError_t (*gauss)(State &s, const void *U, uint32_t *n_partials);
    // one projection sweep E -> E_alt with G -> G_alt (= gauss(E_alt)) and its residual partials
    cudaError_t (*gauss_sweep)(State &s, const void *U, uint32_t *n_partials);
    cudaError_t (*gauss_to_aos)(State &s, double *d_out);
    // the FP64 projection in the adjoint representation (null for the FP32 forms): s.R <- the
    // adjoint matrices of U; G <- the Gauss law's components and residual partials; one step on E
    cudaError_t (*adjoint_links)(State &s, const void *U);
    cudaError_t (*gauss_adj)(State &s, uint32_t *n_partials);
    cudaError_t (*gauss_step_adj)(State &s);
    // plaquette partials (3 rows) of links buffer U, returns #partials
    cudaError_t (*plaquette)(State &s, const void *U, uint32_t *n_partials);
    // partials of sum Re Tr[P(Unew) - P(Uold)]
    cudaError_t (*plaquette_delta)(State &s, const void *Uold, const void *Unew, uint32_t *n_partials);
    cudaError_t (*efield_sumsq)(State &s, const void *E, uint32_t *n_partials);
    // partials (2 rows) of sum (e_new - e_old)(e_new + e_old) and of sum e_old^2 (as efield_sumsq)
    cudaError_t (*efield_sumsq_delta)(State &s, const void *Eold, const void *Enew, uint32_t *n_partials);
    cudaError_t (*normalize)(State &s, void *U);
    // finalize NV rows of n partials into d_out[offset..]
    cudaError_t (*finalize)(State &s, int nv, uint32_t n, int offset);
    // out (an E-field buffer, zeroed) <- scale * Im Tr(T^a U Sigma) per link
    cudaError_t (*force)(State &s, const void *U, void *out, double scale);
    // U_mu(site) <- exp(i angle T^a) U_mu(site)
    cudaError_t (*link_rotate)(State &s, void *U, uint32_t site, int mu, int a, double angle);
    // reverse-mode adjoint of the leap-frog (cotangent arrays hold hi parts only):
    // lamU <- scale Sigma^dag; lamU += coef d/dU sum Im Tr(W U Sigma); adjoint of one drift
    cudaError_t (*adj_init)(State &s, const void *U, void *lamU, double scale);
    cudaError_t (*adj_kick)(State &s, const void *U, const void *lamE, void *lamU, double coef);
    cudaError_t (*adj_drift)(State &s, const void *U, const void *E, void *lamU, void *lamE, double kappa);
    // partials of sum a_i b_i over the hi parts of two E-field arrays
    cudaError_t (*dot)(State &s, const void *a, const void *b, uint32_t *n_partials);
    cudaError_t (*cot_links_to_aos)(State &s, const void *lamU, double *d_aos);
    cudaError_t (*cot_efield_to_aos)(State &s, const void *lamE, double *d_aos);
    // clover field strength F_ij (i < j) and magnetic field per site, double, serde 3x3 layout
    cudaError_t (*clover_fields)(State &s, const void *U, double *f_out, double *b_out);
    // one checkerboard class of a Metropolis (0) / heat-bath (1) sweep, in place
    cudaError_t (*mc_sweep)(State &s, void *U, int alg, int mu, int parity, double beta, uint64_t seed,
                            uint64_t sweep, int n_update, double spread, uint32_t *n_partials);
    // E <- a field in the reference layout that the Gauss projection takes next: hi parts only, lo
    // parts cleared (the projection reads hi and clears lo itself); as efield_from_aos without COMP
    cudaError_t (*efield_hi_from_aos)(State &s, const double *d_aos);
};

const Ops *ops_f64(int dim);
const Ops *ops_f32(int dim);
const Ops *ops_mixed(int dim);

// Step limit of every device-side projection loop (a single state's graph, a batch's) when the
// caller gives none (max_steps <= 0): 1 + 4 * 2500 sweeps, the reference's schedule, so the loop
// always ends (LQ_ERR_NOT_CONVERGED); at 32^4 about 1.4 s of FP32 sweeps.
constexpr int kDefaultProjectionSteps = 10001;

// partial slots needed for V sites (per row), and the rows of the partial buffer
inline uint32_t partial_slots_for(uint32_t V) { return (V + 127) / 128 + 64; }
constexpr int kPartialRows = 3;

} // namespace lq

struct lq_state : public lq::State {};
