// lq_batch.cu -- the extern "C" entry points of batched ensembles (lq_batch_*, include/lqgpu.h).
//
// A batch holds n independent ensembles (lattice side L[e], size[e], beta[e]) of one
// dimension and precision in one set of device arrays; an HMC trajectory of every ensemble
// is one sequence of launches, each covering all ensembles:
//   draw momenta -> Gauss law -> projection sweeps until every ensemble has converged ->
//   leap-frog (kick+drift per step) -> Delta H per ensemble -> Metropolis test on the device.
// The sequence is captured once as a CUDA graph; the projection's data-dependent sweep count
// is a conditional while node whose condition the per-ensemble check kernel sets, so a
// trajectory is one graph launch with no host round trip.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "batch.hpp"
#include "kernels.cuh"
#include "lqgpu.h"
#include "state.hpp"

using lq::Batch;

namespace lq {
void set_last_error(const char *text);

// keys[e] = seed + e, counters = counter, result rows restart at 0 (mode bit 1: keys and
// counters, bit 2: rows)
__global__ void __launch_bounds__(256) k_batch_setup(uint64_t *keys, BatchRun *run, int n_ens, uint64_t seed,
                                                     unsigned long long counter, int mode) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_ens; e += gridDim.x * blockDim.x) {
        if (mode & 1) {
            keys[e] = seed + (uint64_t)e;
            run[e].counter = counter;
        }
        if (mode & 2) run[e].row = 0;
    }
}

} // namespace lq

namespace {

int bfail(cudaError_t e, const char *what, int line) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s (%s) in %s at lq_batch.cu:%d", cudaGetErrorName(e), cudaGetErrorString(e), what,
             line);
    lq::set_last_error(buf);
    (void)cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) return LQ_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return LQ_ERR_NO_DEVICE;
    return LQ_ERR_CUDA;
}

#define BK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t _e = (call);                                                                                       \
        if (_e != cudaSuccess) return bfail(_e, #call, __LINE__);                                                      \
    } while (0)

// ---- kernel timing of eager trajectories
void bprof_flush(Batch &b) {
    for (int i = 0; i < b.prof_n; ++i) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, b.prof_ev[2 * i], b.prof_ev[2 * i + 1]) == cudaSuccess) {
            b.prof_ms += ms;
            ++b.prof_launches;
        } else {
            (void)cudaGetLastError();
        }
    }
    b.prof_n = 0;
}
int bprof_begin(Batch &b) {
    if (!b.prof_on || b.capturing || !b.prof_ev) return -1;
    if (b.prof_n == Batch::kProfPairs) {
        if (cudaStreamSynchronize(b.stream) != cudaSuccess) return -1;
        bprof_flush(b);
    }
    cudaEventRecord(b.prof_ev[2 * b.prof_n], b.stream);
    return b.prof_n;
}
void bprof_end(Batch &b, int slot) {
    if (slot < 0) return;
    cudaEventRecord(b.prof_ev[2 * slot + 1], b.stream);
    b.prof_n = slot + 1;
}
void bprof_free(Batch &b) {
    if (!b.prof_ev) return;
    for (int i = 0; i < 2 * Batch::kProfPairs; ++i) cudaEventDestroy(b.prof_ev[i]);
    delete[] b.prof_ev;
    b.prof_ev = nullptr;
    b.prof_on = 0;
}

// a launch of the trajectory, timed while profiling eager trajectories
#define BKL(call)                                                                                                      \
    do {                                                                                                               \
        const int _slot = bprof_begin(b);                                                                              \
        cudaError_t _e = (call);                                                                                       \
        bprof_end(b, _slot);                                                                                           \
        if (_e != cudaSuccess) return bfail(_e, #call, __LINE__);                                                      \
    } while (0)

#define BCHECK(b)                                                                                                      \
    do {                                                                                                               \
        if (!(b)) return LQ_ERR_INVALID_ARGUMENT;                                                                      \
    } while (0)

int link_update_bits(int link_update) {
    switch (link_update) {
    case LQ_LINK_UPDATE_EXP: return lq::MD_EXP;
    case LQ_LINK_UPDATE_EXP_REUNITARIZE: return lq::MD_EXP | lq::MD_REUNIT;
    default: return 0;
    }
}

void drop_graph(Batch &b) {
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    b.exec = nullptr;
    b.graph = nullptr;
}

void free_batch(Batch *b) {
    if (!b) return;
    drop_graph(*b);
    bprof_free(*b);
    for (int i = 0; i < 3; ++i)
        if (b->U[i]) cudaFree(b->U[i]);
    for (int i = 0; i < 2; ++i) {
        if (b->E[i]) cudaFree(b->E[i]);
        if (b->G[i]) cudaFree(b->G[i]);
    }
    void *dev[] = {b->ens, b->run, b->chunks, b->keys, b->partial, b->done, b->flag, b->results, b->staging};
    for (void *p : dev)
        if (p) cudaFree(p);
    if (b->h_flag) cudaFreeHost(b->h_flag);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete static_cast<lq_batch *>(b);
}

int ensure_staging(Batch &b, size_t bytes) {
    if (b.staging_bytes >= bytes) return LQ_OK;
    if (b.staging) {
        BK(cudaStreamSynchronize(b.stream));
        BK(cudaFree(b.staging));
        b.staging = nullptr;
        b.staging_bytes = 0;
    }
    BK(cudaMalloc(&b.staging, bytes));
    b.staging_bytes = bytes;
    return LQ_OK;
}

int ensure_results(Batch &b, int rows) {
    if (b.result_rows >= rows) return LQ_OK;
    BK(cudaStreamSynchronize(b.stream));
    drop_graph(b); // the graph holds the old pointer
    if (b.results) BK(cudaFree(b.results));
    b.results = nullptr;
    b.result_rows = 0;
    BK(cudaMalloc((void **)&b.results, sizeof(lq::BatchResult) * (size_t)rows * b.n_ens));
    BK(cudaMemsetAsync(b.results, 0, sizeof(lq::BatchResult) * (size_t)rows * b.n_ens, b.stream));
    b.result_rows = rows;
    return LQ_OK;
}

// the kick and drift coefficients of every ensemble for step dt, in the single-lattice path's
// arithmetic (Engine::md): kh = (dt/2) (-sqrt(2/3) / size), dr = sqrt(6) / size * dt
int set_step_coefficients(Batch &b, double dt) {
    if (b.coef_dt == dt) return LQ_OK;
    for (auto &en : b.ens_h) {
        const double ce = -std::sqrt(2.0 / 3.0) / en.size;
        en.kh_d = (dt / 2.0) * ce;
        en.dr_d = std::sqrt(2.0 * 3.0) / en.size * dt;
        en.kh_f = (float)en.kh_d;
        en.dr_f = (float)en.dr_d;
    }
    BK(cudaStreamSynchronize(b.stream));
    BK(cudaMemcpy(b.ens, b.ens_h.data(), sizeof(lq::BatchEns) * b.ens_h.size(), cudaMemcpyHostToDevice));
    b.coef_dt = dt;
    return LQ_OK;
}

// state buffer index of ensemble e (run[e].cur), read back from the device
int state_buffer(Batch &b, int e, int *buf) {
    lq::BatchRun r;
    BK(cudaMemcpyAsync(&r, b.run + e, sizeof(r), cudaMemcpyDeviceToHost, b.stream));
    BK(cudaStreamSynchronize(b.stream));
    *buf = r.cur;
    return LQ_OK;
}

// ---- the trajectory as launches on b.stream (eagerly, or while the stream is captured)
// E roles: E[0] receives the draw and, after an odd number of sweeps, the trajectory's
// momenta; the projected start momenta end in E[1] (every ensemble stops after 1, 5, 9, ...
// sweeps and is skipped in between, so all of them finish in E[1]).
int enqueue_projection_start(Batch &b, int max_steps, cudaGraphConditionalHandle h, int use_handle) {
    BKL(b.ops->normal(b, 0));
    BKL(b.ops->gauss(b, 0, 0));
    BKL(b.ops->sweep(b, 0, 1, 0, 1));
    BKL(b.ops->check(b, 1, max_steps, h, use_handle));
    return LQ_OK;
}
int enqueue_projection_block(Batch &b, int max_steps, cudaGraphConditionalHandle h, int use_handle) {
    BKL(b.ops->sweep(b, 1, 0, 1, 0));
    BKL(b.ops->sweep(b, 0, 1, 0, 1));
    BKL(b.ops->sweep(b, 1, 0, 1, 0));
    BKL(b.ops->sweep(b, 0, 1, 0, 1));
    BKL(b.ops->check(b, 4, max_steps, h, use_handle));
    return LQ_OK;
}
// leap-frog from the state (role 0) with momenta E[1] -> E[0], Delta H, accept
int enqueue_md_accept(Batch &b, double dt, int n, int flags) {
    if (b.comp) {
        // the sweeps updated the hi parts only: the projected field is hi + 0
        const size_t half = b.efield_bytes() / 2;
        BKL(cudaMemsetAsync((char *)b.E[1] + half, 0, half, b.stream));
    }
    // the coefficients of dt are in the ensemble table (set_step_coefficients)
    (void)dt;
    const int KD = lq::MD_KICK | lq::MD_DRIFT | link_update_bits(b.link_update);
    BKL(b.ops->md(b, 0, 1, 1, 0, KD, 0));
    int cur = 1, nxt = 2;
    for (int i = 1; i < n; ++i) {
        BKL(b.ops->md(b, cur, nxt, 0, 0, KD, 1));
        const int t = cur;
        cur = nxt;
        nxt = t;
    }
    BKL(b.ops->md(b, cur, cur, 0, 0, lq::MD_KICK, 0));
    BKL(b.ops->plaquette_delta(b, 0, cur));
    BKL(b.ops->sumsq_delta(b, 1, 0));
    BKL(b.ops->accept(b, cur));
    if (flags & LQ_BATCH_MEASURE_PLAQUETTE) BKL(b.ops->record_plaquette(b));
    return LQ_OK;
}

int run_eager(Batch &b, double dt, int n, int max_steps, int flags) {
    int rc = enqueue_projection_start(b, max_steps, 0, 0);
    if (rc) return rc;
    for (;;) {
        BK(cudaMemcpyAsync(b.h_flag, b.flag, sizeof(int), cudaMemcpyDeviceToHost, b.stream));
        BK(cudaStreamSynchronize(b.stream));
        if (!*b.h_flag) break;
        rc = enqueue_projection_block(b, max_steps, 0, 0);
        if (rc) return rc;
    }
    return enqueue_md_accept(b, dt, n, flags);
}

int capture_inner(Batch &b, double dt, int n, int max_steps, int flags);
int capture(Batch &b, double dt, int n, int max_steps, int flags) {
    // no event records inside the captured graph
    b.capturing = 1;
    const int rc = capture_inner(b, dt, n, max_steps, flags);
    b.capturing = 0;
    return rc;
}
int capture_inner(Batch &b, double dt, int n, int max_steps, int flags) {
    drop_graph(b);
    BK(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t g = nullptr;
    int rc = LQ_OK;
    cudaGraphConditionalHandle h = 0;
    auto abort_capture = [&](int code) {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(b.stream, &junk);
        if (junk) cudaGraphDestroy(junk);
        (void)cudaGetLastError();
        return code;
    };
    {
        cudaStreamCaptureStatus st;
        cudaError_t e = cudaStreamGetCaptureInfo(b.stream, &st, nullptr, &g, nullptr, nullptr, nullptr);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return abort_capture(bfail(e, "conditional handle", __LINE__));
    }
    rc = enqueue_projection_start(b, max_steps, h, 1);
    if (rc) return abort_capture(rc);
    {
        cudaStreamCaptureStatus st;
        const cudaGraphNode_t *deps = nullptr;
        const cudaGraphEdgeData *edges = nullptr;
        size_t ndeps = 0;
        cudaError_t e = cudaStreamGetCaptureInfo(b.stream, &st, nullptr, &g, &deps, &edges, &ndeps);
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, deps, edges, ndeps, &cp);
        if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(b.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e != cudaSuccess) return abort_capture(bfail(e, "conditional node", __LINE__));
        // the loop body: four sweeps and the check, captured from a second stream
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(b.cap_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return abort_capture(bfail(e, "body capture", __LINE__));
        cudaStream_t main_stream = b.stream;
        b.stream = b.cap_stream;
        rc = enqueue_projection_block(b, max_steps, h, 1);
        b.stream = main_stream;
        cudaGraph_t body_out = nullptr;
        e = cudaStreamEndCapture(b.cap_stream, &body_out);
        if (rc) return abort_capture(rc);
        if (e != cudaSuccess) return abort_capture(bfail(e, "body capture end", __LINE__));
    }
    rc = enqueue_md_accept(b, dt, n, flags);
    if (rc) return abort_capture(rc);
    BK(cudaStreamEndCapture(b.stream, &b.graph));
    cudaError_t e = cudaGraphInstantiate(&b.exec, b.graph, 0);
    if (e != cudaSuccess) {
        drop_graph(b);
        return bfail(e, "cudaGraphInstantiate", __LINE__);
    }
    b.g_dt = dt;
    b.g_steps = n;
    b.g_max_gauss = max_steps;
    b.g_flags = flags;
    b.g_link_update = b.link_update;
    return LQ_OK;
}

// ---- autotuner: time each candidate launch shape of a kernel class on the batch's own data
int time_class(Batch &b, int cls, double dt, int reps, float *ms) {
    cudaEvent_t e0, e1;
    BK(cudaEventCreate(&e0));
    BK(cudaEventCreate(&e1));
    int rc = LQ_OK;
    auto launch = [&]() -> cudaError_t {
        switch (cls) {
        case lq::BK_MD: return b.ops->md(b, 0, 1, 1, 0, lq::MD_KICK | lq::MD_DRIFT | link_update_bits(b.link_update), 1);
        case lq::BK_SWEEP: return b.ops->sweep(b, 0, 1, 0, 1);
        case lq::BK_GAUSS: return b.ops->gauss(b, 0, 0);
        case lq::BK_PLAQ_DELTA: return b.ops->plaquette_delta(b, 0, 1);
        case lq::BK_SUMSQ_DELTA: return b.ops->sumsq_delta(b, 1, 0);
        case lq::BK_NORMAL: return b.ops->normal(b, 0);
        case lq::BK_PLAQUETTE: return b.ops->plaquette(b, 0);
        default: return cudaErrorInvalidValue;
        }
    };
    cudaError_t e = launch(); // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, b.stream);
    for (int i = 0; i < reps && e == cudaSuccess; ++i) e = launch();
    if (e == cudaSuccess) e = cudaEventRecord(e1, b.stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e != cudaSuccess) rc = bfail(e, "autotune launch", __LINE__);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / (float)reps;
    return rc;
}

} // namespace

extern "C" {

int lq_batch_create(int dim, int n_ensembles, const int *L, const double *size, const double *beta, int precision,
                    lq_batch **out) {
    if (!out) return LQ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n_ensembles <= 0 || n_ensembles > 65535 || !L || !size || !beta) return LQ_ERR_INVALID_ARGUMENT;
    // per ensemble: the checks of LatticeCyclic::new (src/lattice.rs:190-201) and of the
    // momentum distribution N(0, 0.5 / beta)
    if (dim == 0) return LQ_ERR_ZERO_DIMENSION;
    for (int e = 0; e < n_ensembles; ++e) {
        if (size[e] <= 0.0 || std::isnan(size[e]) || std::isinf(size[e])) return LQ_ERR_NON_POSITIVE_SIZE;
        if (L[e] < 2) return LQ_ERR_DIM_TOO_SMALL;
    }
    if (dim < 2 || dim > 4) return LQ_ERR_UNSUPPORTED_DIM;
    if (precision != LQ_PRECISION_F64 && precision != LQ_PRECISION_MIXED && precision != LQ_PRECISION_F32)
        return LQ_ERR_INVALID_ARGUMENT;
    for (int e = 0; e < n_ensembles; ++e) {
        const double sd = 0.5 / beta[e];
        if (!(sd >= 0.0) || std::isinf(sd)) return LQ_ERR_INVALID_NORMAL;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        (void)cudaGetLastError();
        lq::set_last_error("no CUDA device visible");
        return LQ_ERR_NO_DEVICE;
    }
    lq_batch *b = new (std::nothrow) lq_batch();
    if (!b) return LQ_ERR_OUT_OF_MEMORY;
    b->dim = dim;
    b->n_ens = n_ensembles;
    b->precision = precision;
    b->real_bytes = precision == LQ_PRECISION_F64 ? 8 : 4;
    b->comp = precision == LQ_PRECISION_MIXED ? 1 : 0;
    b->ops = precision == LQ_PRECISION_F64     ? lq::batch_ops_f64(dim)
             : precision == LQ_PRECISION_MIXED ? lq::batch_ops_mixed(dim)
                                               : lq::batch_ops_f32(dim);
    // ensemble table and chunk table
    uint64_t tiles = 0, chunks = 0, links = 0;
    b->ens_h.resize(n_ensembles);
    for (int e = 0; e < n_ensembles; ++e) {
        uint64_t V = 1;
        for (int i = 0; i < dim; ++i) {
            V *= (uint64_t)L[e];
            if (V > (1ull << 28)) {
                free_batch(b);
                return LQ_ERR_INVALID_ARGUMENT;
            }
        }
        lq::BatchEns &en = b->ens_h[e];
        memset(&en, 0, sizeof(en));
        en.V = (uint32_t)V;
        en.L = (uint32_t)L[e];
        uint32_t st = 1;
        for (int i = 0; i < 4; ++i) {
            en.stride[i] = st;
            if (i < dim) st *= (uint32_t)L[e];
        }
        lq::divisor_magic(en.L, en.lm, en.ls);
        en.tile0 = (uint32_t)tiles;
        en.chunk0 = (uint32_t)chunks;
        en.nchunks = (uint32_t)((V + lq::kChunk - 1) / lq::kChunk);
        en.size = size[e];
        en.beta = beta[e];
        en.sd_d = 0.5 / beta[e]; // Engine::efield_normal's standard deviation
        en.sd_f = (float)en.sd_d;
        tiles += (V + 31) / 32;
        chunks += en.nchunks;
        links += V * (uint64_t)dim;
        if (tiles * 32 * (uint64_t)dim * 9 > (1ull << 34)) {
            free_batch(b);
            return LQ_ERR_INVALID_ARGUMENT;
        }
    }
    b->total_tiles = (uint32_t)tiles;
    b->n_chunks = (uint32_t)chunks;
    b->total_links = links;
    std::vector<uint2> chunk_h(chunks);
    for (int e = 0; e < n_ensembles; ++e) {
        const lq::BatchEns &en = b->ens_h[e];
        for (uint32_t k = 0; k < en.nchunks; ++k) chunk_h[en.chunk0 + k] = make_uint2((uint32_t)e, k * lq::kChunk);
    }
    std::vector<lq::BatchRun> run_h(n_ensembles);
    for (auto &r : run_h) memset(&r, 0, sizeof(r));

    int rc = LQ_OK;
    auto alloc = [&](void **p, size_t bytes, int line) {
        if (rc) return;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) rc = bfail(e, "cudaMalloc", line);
    };
    for (int i = 0; i < 3; ++i) alloc(&b->U[i], b->link_bytes(), __LINE__);
    for (int i = 0; i < 2; ++i) {
        alloc(&b->E[i], b->efield_bytes(), __LINE__);
        alloc(&b->G[i], b->gauss_bytes(), __LINE__);
    }
    alloc((void **)&b->ens, sizeof(lq::BatchEns) * n_ensembles, __LINE__);
    alloc((void **)&b->run, sizeof(lq::BatchRun) * n_ensembles, __LINE__);
    alloc((void **)&b->chunks, sizeof(uint2) * chunks, __LINE__);
    alloc((void **)&b->keys, sizeof(uint64_t) * n_ensembles, __LINE__);
    alloc((void **)&b->partial, sizeof(double) * 3 * chunks, __LINE__);
    alloc((void **)&b->done, sizeof(unsigned int), __LINE__);
    alloc((void **)&b->flag, sizeof(int), __LINE__);
    if (!rc) {
        cudaError_t e = cudaMallocHost((void **)&b->h_flag, sizeof(int));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
        // a stream of its own by default: the legacy default stream cannot be captured
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
        b->stream = b->own_stream;
        if (e != cudaSuccess) rc = bfail(e, "batch host resources", __LINE__);
    }
    if (!rc) {
        cudaError_t e = cudaSuccess;
        for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaMemsetAsync(b->U[i], 0, b->link_bytes(), b->stream);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
            e = cudaMemsetAsync(b->E[i], 0, b->efield_bytes(), b->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(b->G[i], 0, b->gauss_bytes(), b->stream);
        }
        if (e == cudaSuccess)
            e = cudaMemsetAsync(b->partial, 0, sizeof(double) * 3 * chunks, b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->done, 0, sizeof(unsigned int), b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->flag, 0, sizeof(int), b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e == cudaSuccess)
            e = cudaMemcpy(b->ens, b->ens_h.data(), sizeof(lq::BatchEns) * n_ensembles, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(b->run, run_h.data(), sizeof(lq::BatchRun) * n_ensembles, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(b->chunks, chunk_h.data(), sizeof(uint2) * chunks, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = bfail(e, "batch initialisation", __LINE__);
    }
    if (!rc) {
        for (int e = 0; e < n_ensembles && !rc; ++e) {
            cudaError_t err = b->ops->links_cold(*b, e, 0);
            if (err != cudaSuccess) rc = bfail(err, "links_cold", __LINE__);
        }
    }
    if (!rc) {
        lq::k_batch_setup<<<1, 256, 0, b->stream>>>(b->keys, b->run, n_ensembles, 0, 0, 3);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) rc = bfail(e, "batch setup", __LINE__);
    }
    if (rc) {
        free_batch(b);
        return rc;
    }
    *out = b;
    return LQ_OK;
}

int lq_batch_destroy(lq_batch *b) {
    if (!b) return LQ_OK;
    cudaStreamSynchronize(b->stream);
    free_batch(b);
    return LQ_OK;
}

int lq_batch_set_stream(lq_batch *b, void *stream) {
    BCHECK(b);
    BK(cudaStreamSynchronize(b->stream));
    b->stream = stream ? (cudaStream_t)stream : b->own_stream;
    return LQ_OK;
}

int lq_batch_info(const lq_batch *b, int *dim, int *n_ensembles, long long *total_links, size_t *device_bytes) {
    BCHECK(b);
    if (dim) *dim = b->dim;
    if (n_ensembles) *n_ensembles = b->n_ens;
    if (total_links) *total_links = (long long)b->total_links;
    if (device_bytes)
        *device_bytes = 3 * b->link_bytes() + 2 * b->efield_bytes() + 2 * b->gauss_bytes() +
                        sizeof(double) * 3 * (size_t)b->n_chunks +
                        sizeof(uint2) * (size_t)b->n_chunks +
                        (sizeof(lq::BatchEns) + sizeof(lq::BatchRun) + 8) * (size_t)b->n_ens;
    return LQ_OK;
}

int lq_batch_set_link_update(lq_batch *b, int link_update) {
    BCHECK(b);
    if (link_update != LQ_LINK_UPDATE_EULER && link_update != LQ_LINK_UPDATE_EXP &&
        link_update != LQ_LINK_UPDATE_EXP_REUNITARIZE)
        return LQ_ERR_INVALID_ARGUMENT;
    b->link_update = link_update;
    return LQ_OK;
}

int lq_batch_set_seed(lq_batch *b, uint64_t seed, uint64_t counter) {
    BCHECK(b);
    lq::k_batch_setup<<<1, 256, 0, b->stream>>>(b->keys, b->run, b->n_ens, seed, counter, 1);
    BK(cudaGetLastError());
    BK(cudaStreamSynchronize(b->stream));
    b->seed = seed;
    return LQ_OK;
}

int lq_batch_links_random(lq_batch *b, uint64_t seed) {
    BCHECK(b);
    for (int e = 0; e < b->n_ens; ++e) {
        int buf = 0;
        int rc = state_buffer(*b, e, &buf);
        if (rc) return rc;
        BK(b->ops->links_random(*b, e, buf, seed + (uint64_t)e));
    }
    BK(cudaStreamSynchronize(b->stream));
    return LQ_OK;
}

int lq_batch_links_upload(lq_batch *b, int ensemble, const double *links, size_t n) {
    BCHECK(b);
    if (ensemble < 0 || ensemble >= b->n_ens || !links) return LQ_ERR_INVALID_ARGUMENT;
    const size_t want = (size_t)b->ens_h[ensemble].V * b->dim * 18;
    if (n != want) return LQ_ERR_INCOMPATIBLE_SIZE;
    int rc = ensure_staging(*b, n * sizeof(double));
    if (rc) return rc;
    int buf = 0;
    rc = state_buffer(*b, ensemble, &buf);
    if (rc) return rc;
    BK(cudaMemcpyAsync(b->staging, links, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    BK(b->ops->links_from_aos(*b, ensemble, buf, (const double *)b->staging));
    BK(cudaStreamSynchronize(b->stream));
    return LQ_OK;
}

int lq_batch_links_download(lq_batch *b, int ensemble, double *links, size_t n) {
    BCHECK(b);
    if (ensemble < 0 || ensemble >= b->n_ens || !links) return LQ_ERR_INVALID_ARGUMENT;
    const size_t want = (size_t)b->ens_h[ensemble].V * b->dim * 18;
    if (n != want) return LQ_ERR_INCOMPATIBLE_SIZE;
    int rc = ensure_staging(*b, n * sizeof(double));
    if (rc) return rc;
    int buf = 0;
    rc = state_buffer(*b, ensemble, &buf);
    if (rc) return rc;
    BK(b->ops->links_to_aos(*b, ensemble, buf, (double *)b->staging));
    BK(cudaMemcpyAsync(links, b->staging, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    return LQ_OK;
}

int lq_batch_normalize_link_matrices(lq_batch *b) {
    BCHECK(b);
    for (int e = 0; e < b->n_ens; ++e) {
        int buf = 0;
        int rc = state_buffer(*b, e, &buf);
        if (rc) return rc;
        BK(b->ops->normalize(*b, e, buf));
    }
    BK(cudaStreamSynchronize(b->stream));
    return LQ_OK;
}

int lq_batch_average_trace_plaquette(lq_batch *b, double *re, double *im) {
    BCHECK(b);
    const size_t bytes = sizeof(double) * 3 * (size_t)b->n_ens;
    int rc = ensure_staging(*b, bytes);
    if (rc) return rc;
    BK(b->ops->plaquette_sums(*b, (double *)b->staging));
    std::vector<double> sums(3 * (size_t)b->n_ens);
    BK(cudaMemcpyAsync(sums.data(), b->staging, bytes, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (int e = 0; e < b->n_ens; ++e) {
        const double n_plaq = (double)((uint64_t)b->ens_h[e].V * (uint64_t)((b->dim * (b->dim - 1)) / 2));
        if (re) re[e] = sums[3 * (size_t)e + 1] / n_plaq;
        if (im) im[e] = sums[3 * (size_t)e + 2] / n_plaq;
    }
    return LQ_OK;
}

int lq_batch_autotune(lq_batch *b, double dt, int reps) {
    BCHECK(b);
    if (reps <= 0 || !(dt > 0.0)) return LQ_ERR_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    BK(cudaGetDevice(&dev));
    BK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    BK(cudaStreamSynchronize(b->stream));
    drop_graph(*b);
    int rc0 = set_step_coefficients(*b, dt);
    if (rc0) return rc0;
    // inputs for the timed launches: a fresh draw and its Gauss law (E is scratch between
    // trajectories; the state's links are only read)
    BK(b->ops->normal(*b, 0));
    BK(b->ops->gauss(*b, 0, 0));
    for (int cls = 0; cls < lq::BK_CLASSES; ++cls) {
        const bool per_link = cls == lq::BK_MD || cls == lq::BK_NORMAL;
        const uint32_t n_work = b->n_chunks * (per_link ? (uint32_t)b->dim : 1u);
        const int occ = b->ops->occupancy(cls);
        std::vector<uint32_t> grids = {0};
        if (occ > 0)
            for (uint32_t m : {1u, 2u, 4u, 8u}) {
                const uint32_t g = (uint32_t)sms * (uint32_t)occ * m;
                if (g < n_work) grids.push_back(g);
            }
        lq::Shape best;
        best.ms = -1.0f;
        for (int order = 0; order < (per_link ? 2 : 1); ++order)
            for (uint32_t g : grids) {
                b->shape[cls].grid = g;
                b->shape[cls].order = order;
                float ms = 0.0f;
                int rc = time_class(*b, cls, dt, reps, &ms);
                if (rc) return rc;
                if (best.ms < 0.0f || ms < best.ms) {
                    best.grid = g;
                    best.order = order;
                    best.ms = ms;
                }
            }
        b->shape[cls] = best;
    }
    return LQ_OK;
}

int lq_batch_tuning(const lq_batch *b, int kernel_class, int *grid, int *order, double *ms) {
    BCHECK(b);
    if (kernel_class < 0 || kernel_class >= lq::BK_CLASSES) return LQ_ERR_INVALID_ARGUMENT;
    const lq::Shape &s = b->shape[kernel_class];
    if (grid) *grid = (int)s.grid;
    if (order) *order = s.order;
    if (ms) *ms = s.ms;
    return LQ_OK;
}

int lq_batch_hmc_run(lq_batch *b, double dt, int n_steps, int n_trajectories, int max_gauss_steps, int flags) {
    BCHECK(b);
    if (n_steps <= 0) return LQ_ERR_ZERO_INTEGRATION;
    if (n_trajectories <= 0 || (flags & ~(LQ_BATCH_USE_GRAPH | LQ_BATCH_MEASURE_PLAQUETTE)))
        return LQ_ERR_INVALID_ARGUMENT;
    const int max_steps = max_gauss_steps > 0 ? max_gauss_steps : lq::kDefaultProjectionSteps;
    int rc = ensure_results(*b, n_trajectories);
    if (!rc) rc = set_step_coefficients(*b, dt);
    if (rc) return rc;
    lq::k_batch_setup<<<1, 256, 0, b->stream>>>(b->keys, b->run, b->n_ens, 0, 0, 2);
    BK(cudaGetLastError());
    if (flags & LQ_BATCH_USE_GRAPH) {
        const int gflags = flags & LQ_BATCH_MEASURE_PLAQUETTE;
        if (!b->exec || b->g_dt != dt || b->g_steps != n_steps || b->g_max_gauss != max_steps ||
            b->g_flags != gflags || b->g_link_update != b->link_update) {
            rc = capture(*b, dt, n_steps, max_steps, gflags);
            if (rc) return rc;
        }
        for (int k = 0; k < n_trajectories; ++k) {
            BK(cudaGraphLaunch(b->exec, b->stream));
            ++b->graph_launches;
        }
    } else {
        for (int k = 0; k < n_trajectories; ++k) {
            rc = run_eager(*b, dt, n_steps, max_steps, flags);
            if (rc) return rc;
        }
    }
    BK(cudaStreamSynchronize(b->stream));
    return LQ_OK;
}

int lq_batch_hmc_results(lq_batch *b, int first, int count, double *delta_h, double *prob, double *uniform,
                         int *accepted, int *gauss_steps, int *status, double *plaquette) {
    BCHECK(b);
    if (first < 0 || count <= 0 || first + count > b->result_rows) return LQ_ERR_INVALID_ARGUMENT;
    std::vector<lq::BatchResult> rows((size_t)count * b->n_ens);
    BK(cudaMemcpyAsync(rows.data(), b->results + (size_t)first * b->n_ens, sizeof(lq::BatchResult) * rows.size(),
                       cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < rows.size(); ++i) {
        const lq::BatchResult &r = rows[i];
        if (delta_h) delta_h[i] = r.delta_h;
        if (prob) prob[i] = r.prob;
        if (uniform) uniform[i] = r.uniform;
        if (accepted) accepted[i] = r.accepted;
        if (gauss_steps) gauss_steps[i] = r.gauss_steps;
        if (status) status[i] = r.status;
        if (plaquette) plaquette[i] = r.plaq_re;
    }
    return LQ_OK;
}

int lq_batch_profile_enable(lq_batch *b, int on) {
    BCHECK(b);
    if (on && !b->prof_ev) {
        b->prof_ev = new (std::nothrow) cudaEvent_t[2 * Batch::kProfPairs];
        if (!b->prof_ev) return LQ_ERR_OUT_OF_MEMORY;
        for (int i = 0; i < 2 * Batch::kProfPairs; ++i) {
            const cudaError_t e = cudaEventCreate(&b->prof_ev[i]);
            if (e != cudaSuccess) {
                for (int j = 0; j < i; ++j) cudaEventDestroy(b->prof_ev[j]);
                delete[] b->prof_ev;
                b->prof_ev = nullptr;
                return bfail(e, "cudaEventCreate", __LINE__);
            }
        }
    }
    if (!on) {
        BK(cudaStreamSynchronize(b->stream));
        bprof_flush(*b);
        bprof_free(*b);
    }
    b->prof_on = on ? 1 : 0;
    return LQ_OK;
}

int lq_batch_profile_read(lq_batch *b, long long *launches, double *kernel_ms, int reset) {
    BCHECK(b);
    BK(cudaStreamSynchronize(b->stream));
    if (b->prof_ev) bprof_flush(*b);
    if (launches) *launches = b->prof_launches;
    if (kernel_ms) *kernel_ms = b->prof_ms;
    if (reset) {
        b->prof_launches = 0;
        b->prof_ms = 0.0;
    }
    return LQ_OK;
}

int lq_batch_graph_launches(const lq_batch *b, long long *launches) {
    BCHECK(b);
    if (!launches) return LQ_ERR_INVALID_ARGUMENT;
    *launches = b->graph_launches;
    return LQ_OK;
}

} // extern "C"
