// batch.hpp -- many independent HMC ensembles of uneven lattice size and beta held in one
// set of device arrays (the lq_batch handle), and the per-(D, precision) table of batched
// device operations.
//
// Layout: the ensembles' tiled arrays are concatenated tile by tile.  Ensemble e owns tiles
// [tile0, tile0 + tiles_of(V)) of every array, so with its base offset (tile0 * planes * 32
// elements) the single-lattice index tix(site, planes, plane) addresses it unchanged; the lo
// arrays of compensated storage follow the hi arrays of the whole batch.  Work is split into
// chunks of 128 consecutive sites of one ensemble (the last chunk of an ensemble may be
// partial); a kernel walks the table of chunks (x D directions for per-link kernels), so one
// launch covers every ensemble, and reductions leave one partial per chunk, summed per
// ensemble in a fixed order: results do not depend on the launch shape.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "lqgpu.h"

namespace lq {

constexpr uint32_t kChunk = 128; // sites per chunk = threads per block of the batched kernels

// per ensemble, constant after creation (device copy)
struct BatchEns {
    uint32_t V, L, tile0, chunk0, nchunks, ls;
    uint32_t stride[4];
    uint32_t lm, pad; // division by L (divisor_magic: multiplier lm, shift ls)
    double size, beta;
    // coefficients in the single-lattice path's arithmetic (Engine::md, Engine::efield_normal),
    // computed on the host in double and stored in both storage types so that no kernel needs
    // FP64 arithmetic per work item: momentum std dev 0.5 / beta, half kick (dt/2) c_e with
    // c_e = -sqrt(2/3) / size, drift dt sqrt(6) / size (kh, dr follow the dt of the last run)
    double sd_d, kh_d, dr_d;
    float sd_f, kh_f, dr_f, pad_f;
};

// per ensemble, updated on the device by the trajectory kernels
struct BatchRun {
    int cur;                    // link buffer (0..2) holding the state
    int converged;              // the projection of this trajectory has finished (or failed)
    int steps;                  // projection steps of this trajectory
    int status;                 // LQ_OK, LQ_ERR_GAUSS_PROJECTION or LQ_ERR_NOT_CONVERGED
    unsigned long long counter; // Philox counter of the next trajectory (trajectories run)
    int row;                    // result row of the next trajectory of the current run
    int pad;
};

// one trajectory of one ensemble (lq_batch_hmc_results)
struct BatchResult {
    double delta_h, prob, uniform, plaq_re, plaq_im;
    int accepted, gauss_steps, status, pad;
};

// kernel classes with a tuned launch shape
enum : int {
    BK_MD = 0,
    BK_SWEEP,
    BK_GAUSS,
    BK_PLAQ_DELTA,
    BK_SUMSQ_DELTA,
    BK_NORMAL,
    BK_PLAQUETTE,
    BK_CLASSES
};

// launch shape of one kernel class: grid blocks (0: one block per work item) and the work
// order of per-link kernels (0: directions fastest, 1: chunks fastest)
struct Shape {
    uint32_t grid = 0;
    int order = 0;
    float ms = 0.0f; // measured by the autotuner (0: not tuned)
};

struct BatchOps;

struct Batch {
    int dim = 0;
    int n_ens = 0;
    int precision = LQ_PRECISION_MIXED;
    size_t real_bytes = 4;
    int comp = 0;
    int link_update = LQ_LINK_UPDATE_EULER;
    cudaStream_t stream = nullptr;
    std::vector<BatchEns> ens_h;
    uint32_t total_tiles = 0;
    uint32_t n_chunks = 0;
    uint64_t total_links = 0;

    void *U[3] = {nullptr, nullptr, nullptr};
    void *E[2] = {nullptr, nullptr};
    void *G[2] = {nullptr, nullptr};
    BatchEns *ens = nullptr;
    BatchRun *run = nullptr;
    uint2 *chunks = nullptr;    // {ensemble, first site}
    uint64_t *keys = nullptr;   // Philox key of each ensemble
    double *partial = nullptr;  // 3 rows of n_chunks
    unsigned int *done = nullptr; // last-block counter of the per-ensemble kernels
    int *flag = nullptr;          // device: 1 while a projection is unfinished
    int *h_flag = nullptr;        // pinned host mirror
    BatchResult *results = nullptr;
    int result_rows = 0;
    uint64_t seed = 0;
    void *staging = nullptr; // f64 AoS staging for per-ensemble uploads / downloads
    size_t staging_bytes = 0;

    Shape shape[BK_CLASSES];

    // the captured trajectory and what it was captured for
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap_stream = nullptr; // stream used to capture the projection loop body
    cudaStream_t own_stream = nullptr; // the batch's stream unless lq_batch_set_stream names one
    double coef_dt = -1.0; // dt of the kh / dr coefficients in the ensemble table
    double g_dt = 0.0;
    int g_steps = 0, g_max_gauss = 0, g_flags = 0, g_link_update = -1;
    long long graph_launches = 0;

    // kernel time of eagerly launched trajectories (lq_batch_profile_enable): an event pair around
    // every launch, summed at each synchronisation; never inside a capture
    static constexpr int kProfPairs = 512;
    int prof_on = 0;
    int capturing = 0;
    cudaEvent_t *prof_ev = nullptr; // 2 * kProfPairs events while profiling is enabled
    int prof_n = 0;
    long long prof_launches = 0;
    double prof_ms = 0.0;

    const BatchOps *ops = nullptr;

    size_t link_elems() const { return (size_t)total_tiles * 32 * dim * 9; }
    size_t link_bytes() const { return link_elems() * 2 * real_bytes * (comp ? 2 : 1); }
    size_t efield_elems() const { return (size_t)total_tiles * 32 * dim * 8; }
    size_t efield_bytes() const { return efield_elems() * real_bytes * (comp ? 2 : 1); }
    size_t gauss_bytes() const { return (size_t)total_tiles * 32 * 9 * real_bytes; }
};

// Batched device operations of one (D, T, COMP) instantiation, asynchronous on b.stream.
// Link buffer roles r are relative to each ensemble's state buffer: U[(cur + r) % 3].
struct BatchOps {
    // one ensemble e, link buffer buf (its state buffer): AoS f64 <-> device, initial links
    cudaError_t (*links_from_aos)(Batch &b, int e, int buf, const double *d_aos);
    cudaError_t (*links_to_aos)(Batch &b, int e, int buf, double *d_aos);
    cudaError_t (*links_random)(Batch &b, int e, int buf, uint64_t seed);
    cudaError_t (*links_cold)(Batch &b, int e, int buf);
    cudaError_t (*normalize)(Batch &b, int e, int buf);
    // trajectory kernels over every ensemble
    cudaError_t (*normal)(Batch &b, int eout);
    cudaError_t (*gauss)(Batch &b, int ein, int gout);
    cudaError_t (*sweep)(Batch &b, int ein, int eout, int gin, int gout);
    cudaError_t (*check)(Batch &b, int steps_added, int max_steps, cudaGraphConditionalHandle h, int use_handle);
    // kick (k1 = kh when k1_on, else 0; k2 = kh) and drift with the coefficients of the table
    cudaError_t (*md)(Batch &b, int rin, int rout, int ein, int eout, int mode, int k1_on);
    cudaError_t (*plaquette_delta)(Batch &b, int r_old, int r_new);
    cudaError_t (*sumsq_delta)(Batch &b, int e_old, int e_new);
    cudaError_t (*accept)(Batch &b, int r_final);
    cudaError_t (*plaquette)(Batch &b, int role);
    // per-ensemble plaquette sums of the state into out[3 * e + {0, 1, 2}] (device doubles)
    cudaError_t (*plaquette_sums)(Batch &b, double *d_out);
    cudaError_t (*record_plaquette)(Batch &b);
    // resident blocks per SM of a kernel class (for the autotuner's persistent grids)
    int (*occupancy)(int cls);
};

const BatchOps *batch_ops_f64(int dim);
const BatchOps *batch_ops_f32(int dim);
const BatchOps *batch_ops_mixed(int dim);

} // namespace lq

struct lq_batch : public lq::Batch {};
