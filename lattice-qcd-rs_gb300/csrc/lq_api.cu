// lq_api.cu -- the extern "C" entry points declared in include/lqgpu.h.
//
// Host orchestration of the device state: validation with the reference's error
// taxonomy, buffer management, the integrator schedules and the HMC trajectory.  All
// device work is enqueued on the state's stream; functions that hand a value back to the
// host synchronise that stream once.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "kernels.cuh"
#include "lqgpu.h"
#include "state.hpp"
#include "sweeps.cuh"

using lq::State;

#ifndef LQ_BLOCK_REUSE_SITES
#define LQ_BLOCK_REUSE_SITES 32768
#endif

namespace lq {
namespace {
using BoundsReader = int (*)(unsigned long long *, unsigned long long *, int);
std::vector<BoundsReader> &bounds_readers() {
    static std::vector<BoundsReader> r; // filled during static initialisation of the library
    return r;
}
} // namespace
int register_bounds_reader(BoundsReader read) {
    bounds_readers().push_back(read);
    return 0;
}
} // namespace lq

namespace {

thread_local std::string g_last_error;

int cuda_fail(cudaError_t e, const char *what, int line) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s (%s) in %s at lq_api.cu:%d", cudaGetErrorName(e), cudaGetErrorString(e), what,
             line);
    g_last_error = buf;
    (void)cudaGetLastError(); // clear a non-sticky error so the context stays usable
    if (e == cudaErrorMemoryAllocation) return LQ_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return LQ_ERR_NO_DEVICE;
    return LQ_ERR_CUDA;
}

#define LQ_CK(call)                                                                                                    \
    do {                                                                                                               \
        cudaError_t _e = (call);                                                                                       \
        if (_e != cudaSuccess) return cuda_fail(_e, #call, __LINE__);                                                  \
    } while (0)

#define LQ_LAUNCH(st, cls, call)                                                                                       \
    do {                                                                                                               \
        const int _slot = prof_begin(st, cls);                                                                         \
        cudaError_t _e = (call);                                                                                       \
        prof_end(st, _slot, cls);                                                                                      \
        if (_e != cudaSuccess) return cuda_fail(_e, #call, __LINE__);                                                  \
    } while (0)

#define LQ_CHECK_STATE(s)                                                                                              \
    do {                                                                                                               \
        if (!(s)) return LQ_ERR_INVALID_ARGUMENT;                                                                      \
    } while (0)

// ---- launch counters: an event pair around every launch while profiling is enabled
void prof_flush(State &s) {
    lq::Prof *p = s.prof;
    if (!p) return;
    for (int i = 0; i < p->n; ++i) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, p->ev[2 * i], p->ev[2 * i + 1]) == cudaSuccess) {
            p->ms[p->cls[i]] += ms;
            p->launches[p->cls[i]] += p->cnt[i];
        } else {
            (void)cudaGetLastError();
        }
    }
    p->n = 0;
}
cudaError_t sync_stream(State &s) {
    cudaError_t e = cudaStreamSynchronize(s.stream);
    if (e == cudaSuccess) prof_flush(s);
    return e;
}
int prof_begin(State &s, int cls) {
    lq::Prof *p = s.prof;
    if (!p || !((s.prof_mask >> cls) & 1u)) return -1;
    if (p->n == lq::kProfPool) {
        if (cudaStreamSynchronize(s.stream) != cudaSuccess) return -1;
        prof_flush(s);
    }
    cudaEventRecord(p->ev[2 * p->n], s.stream);
    return p->n;
}
void prof_end(State &s, int slot, int cls) {
    lq::Prof *p = s.prof;
    if (!p || slot < 0) return;
    cudaEventRecord(p->ev[2 * slot + 1], s.stream);
    p->cls[slot] = cls;
    p->cnt[slot] = 1;
    p->n = slot + 1;
}
void prof_free(State &s) {
    if (!s.prof) return;
    for (int i = 0; i < 2 * lq::kProfPool; ++i) cudaEventDestroy(s.prof->ev[i]);
    delete s.prof;
    s.prof = nullptr;
}

// machine epsilon of the arithmetic of the state (the projection residual floor follows it)
double eps_of(const State &s) { return s.precision == LQ_PRECISION_F64 ? 2.220446049250313e-16 : 1.1920928955078125e-07; }

void free_state(State *s) {
    if (!s) return;
    prof_free(*s);
    for (int i = 0; i < 3; ++i)
        if (s->U[i]) cudaFree(s->U[i]);
    if (s->E) cudaFree(s->E);
    if (s->E_alt) cudaFree(s->E_alt);
    if (s->G) cudaFree(s->G);
    if (s->G_alt) cudaFree(s->G_alt);
    if (s->R) cudaFree(s->R);
    if (s->partial) cudaFree(s->partial);
    if (s->d_out) cudaFree(s->d_out);
    if (s->h_out) cudaFreeHost(s->h_out);
    if (s->staging) cudaFree(s->staging);
    if (s->prefetch) cudaFree(s->prefetch);
    if (s->prefetch_done) cudaEventDestroy(s->prefetch_done);
    if (s->prefetch_free) cudaEventDestroy(s->prefetch_free);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    for (int i = 0; i < s->n_proj; ++i)
        if (s->proj[i].exec) cudaGraphExecDestroy(s->proj[i].exec);
    if (s->d_proj) cudaFree(s->d_proj);
    if (s->cap_main) cudaStreamDestroy(s->cap_main);
    if (s->cap_body) cudaStreamDestroy(s->cap_body);
    delete static_cast<lq_state *>(s);
}

int ensure_staging(State &s, size_t bytes) {
    if (s.staging_bytes >= bytes) return LQ_OK;
    if (s.staging) {
        LQ_CK(sync_stream(s));
        LQ_CK(cudaFree(s.staging));
        s.staging = nullptr;
        s.staging_bytes = 0;
    }
    LQ_CK(cudaMalloc(&s.staging, bytes));
    s.staging_bytes = bytes;
    return LQ_OK;
}

void state_changed(State &s) {
    s.hu_valid = 0;
    s.has_pending = 0;
    s.pending_buf = -1;
}

int other_buffer(const State &s, int avoid1, int avoid2) {
    for (int i = 0; i < 3; ++i)
        if (i != avoid1 && i != avoid2) return i;
    return -1;
}

// d_out[offset..offset+2] <- plaquette sums of links buffer U
int plaquette_sums(State &s, const void *U, int offset) {
    uint32_t n = 0;
    LQ_LAUNCH(s, LQ_KERNEL_PLAQUETTE, s.ops->plaquette(s, U, &n));
    LQ_LAUNCH(s, LQ_KERNEL_REDUCE, s.ops->finalize(s, 3, n, offset));
    return LQ_OK;
}
// d_out[offset] <- sum of e^2 of the current E-field
int efield_sumsq(State &s, int offset) {
    uint32_t n = 0;
    LQ_LAUNCH(s, LQ_KERNEL_REDUCE, s.ops->efield_sumsq(s, s.E, &n));
    LQ_LAUNCH(s, LQ_KERNEL_REDUCE, s.ops->finalize(s, 1, n, offset));
    return LQ_OK;
}
int fetch_out(State &s, int count) {
    LQ_CK(cudaMemcpyAsync(s.h_out, s.d_out, sizeof(double) * count, cudaMemcpyDeviceToHost, s.stream));
    LQ_CK(sync_stream(s));
    return LQ_OK;
}

// symplectic_n from U[src] (kept) into the other two buffers; returns the final buffer index.
// E <- E + dt/2 F(U_k) (+ dt/2 F(U_k) of the next step) ...; U_{k+1} = U_k + dt dU(E, U_k).
// With e_to_alt the first kick reads s.E and writes s.E_alt (later steps update s.E_alt in
// place), so the start momenta survive in s.E.
int link_update_bits(int link_update) {
    switch (link_update) {
    case LQ_LINK_UPDATE_EXP: return lq::MD_EXP;
    case LQ_LINK_UPDATE_EXP_REUNITARIZE: return lq::MD_EXP | lq::MD_REUNIT;
    default: return 0;
    }
}

int run_symplectic(State &s, int src, double dt, int n, bool e_to_alt, int link_update, int *final_buf) {
    const int a = other_buffer(s, src, -1);
    const int b = other_buffer(s, src, a);
    void *ew = e_to_alt ? s.E_alt : s.E;
    const int KD = lq::MD_KICK | lq::MD_DRIFT | link_update_bits(link_update);
    LQ_LAUNCH(s, LQ_KERNEL_MD, s.ops->md(s, s.U[src], s.U[a], s.E, ew, KD, 0.0, dt / 2.0, dt));
    int cur = a, nxt = b;
    for (int i = 1; i < n; ++i) {
        LQ_LAUNCH(s, LQ_KERNEL_MD, s.ops->md(s, s.U[cur], s.U[nxt], ew, ew, KD, dt / 2.0, dt / 2.0, dt));
        const int t = cur;
        cur = nxt;
        nxt = t;
    }
    LQ_LAUNCH(s, LQ_KERNEL_MD, s.ops->md(s, s.U[cur], s.U[cur], ew, ew, lq::MD_KICK, 0.0, dt / 2.0, 0.0));
    *final_buf = cur;
    return LQ_OK;
}

// The projection's convergence test on the device, a node of the projection graph: the residual
// partials are summed exactly as k_finalize<1> sums them (so the value equals the host loop's),
// the sweeps since the last test are added to ctl[0], and the loop condition is set as the host
// loop decides: stop on NaN (ctl[1] = LQ_ERR_GAUSS_PROJECTION), at or below the threshold, or
// when four more sweeps would pass the step limit (ctl[1] = LQ_ERR_NOT_CONVERGED).
__global__ void __launch_bounds__(1024) k_proj_check(const double *__restrict__ partial, uint32_t n, double threshold,
                                                     int steps_added, int max_steps, int *ctl,
                                                     cudaGraphConditionalHandle h) {
    double v[1] = {0.0};
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) v[0] += partial[k];
    __shared__ double res[1];
    lq::block_reduce_store<1>(v, res, 0, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        const int steps = ctl[0] + steps_added;
        ctl[0] = steps;
        const double val = res[0];
        unsigned int go = 0;
        if (isnan(val)) ctl[1] = LQ_ERR_GAUSS_PROJECTION;
        else if (val <= threshold) ctl[1] = LQ_OK;
        else if (max_steps > 0 && steps + 4 > max_steps) ctl[1] = LQ_ERR_NOT_CONVERGED;
        else go = 1;
        cudaGraphSetConditional(h, go);
    }
}

double projection_threshold(const State &s) { return eps_of(s) * (double)((uint64_t)s.V * 4 * 8 * 10); }

// Captures the sweep loop of project_gauss for the current link buffer, E/G buffer order and step
// limit: Gauss law, one sweep, the test, then a while node whose body is four sweeps and the
// test.  Every run makes 1 + 4k sweeps, so each body leaves E/G in the buffers the first sweep
// wrote and the baked pointers stay valid for every iteration; the capture itself enqueues (and
// so swaps the state's E/G pointers) five times, and the order is restored at the end.
int capture_projection(State &s, int max_steps, cudaGraphExec_t *out) {
    *out = nullptr;
    if (!s.d_proj) LQ_CK(cudaMalloc((void **)&s.d_proj, 4 * sizeof(int)));
    if (!s.cap_main) LQ_CK(cudaStreamCreateWithFlags(&s.cap_main, cudaStreamNonBlocking));
    if (!s.cap_body) LQ_CK(cudaStreamCreateWithFlags(&s.cap_body, cudaStreamNonBlocking));
    const void *U = s.U[s.cur];
    const double threshold = projection_threshold(s);
    void *E0 = s.E, *E1 = s.E_alt, *G0 = s.G, *G1 = s.G_alt;
    const cudaStream_t user_stream = s.stream;
    s.stream = s.cap_main;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s.cap_main, cudaStreamCaptureModeThreadLocal);
    bool capturing = e == cudaSuccess;
    cudaGraphConditionalHandle h = 0;
    uint32_t n = 0;
    // FP32 forms: one fused sweep, double-buffered; FP64: the step in place and the Gauss law on the
    // links' transport tables
    const bool fused = s.precision != LQ_PRECISION_F64;
    auto sweep = [&]() {
        if (!fused) {
            cudaError_t r = s.ops->gauss_step_adj(s);
            return r == cudaSuccess ? s.ops->gauss_adj(s, &n) : r;
        }
        cudaError_t r = s.ops->gauss_sweep(s, U, &n);
        std::swap(s.E, s.E_alt);
        std::swap(s.G, s.G_alt);
        return r;
    };
    if (e == cudaSuccess) {
        cudaStreamCaptureStatus st;
        e = cudaStreamGetCaptureInfo(s.cap_main, &st, nullptr, &g, nullptr, nullptr, nullptr);
    }
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.d_proj, 0, 4 * sizeof(int), s.stream);
    if (e == cudaSuccess) e = fused ? s.ops->gauss(s, U, &n) : s.ops->adjoint_links(s, U);
    if (e == cudaSuccess && !fused) e = s.ops->gauss_adj(s, &n);
    if (e == cudaSuccess) e = sweep();
    if (e == cudaSuccess) {
        k_proj_check<<<1, 1024, 0, s.stream>>>(s.partial, n, threshold, 1, max_steps, s.d_proj, h);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        cudaStreamCaptureStatus st;
        const cudaGraphNode_t *deps = nullptr;
        const cudaGraphEdgeData *edges = nullptr;
        size_t ndeps = 0;
        e = cudaStreamGetCaptureInfo(s.cap_main, &st, nullptr, &g, &deps, &edges, &ndeps);
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, deps, edges, ndeps, &cp);
        if (e == cudaSuccess)
            e = cudaStreamUpdateCaptureDependencies(s.cap_main, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e == cudaSuccess) {
            e = cudaStreamBeginCaptureToGraph(s.cap_body, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                s.stream = s.cap_body;
                for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = sweep();
                if (e == cudaSuccess) {
                    k_proj_check<<<1, 1024, 0, s.stream>>>(s.partial, n, threshold, 4, max_steps, s.d_proj, h);
                    e = cudaGetLastError();
                }
                cudaGraph_t body = nullptr;
                const cudaError_t e2 = cudaStreamEndCapture(s.cap_body, &body);
                if (e == cudaSuccess) e = e2;
            }
        }
    }
    cudaGraph_t graph = nullptr;
    if (capturing) {
        const cudaError_t e2 = cudaStreamEndCapture(s.cap_main, &graph);
        if (e == cudaSuccess) e = e2;
    }
    s.stream = user_stream;
    s.E = E0;
    s.E_alt = E1;
    s.G = G0;
    s.G_alt = G1;
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        *out = nullptr;
        return cuda_fail(e, "projection graph capture", __LINE__);
    }
    return LQ_OK;
}

// project_gauss through the captured graph: one launch and one read of (sweeps, status)
int project_gauss_graph(State &s, int max_steps, int *steps_done) {
    if (max_steps <= 0) max_steps = lq::kDefaultProjectionSteps;
    const void *U = s.U[s.cur];
    cudaGraphExec_t exec = nullptr;
    for (int i = 0; i < s.n_proj; ++i) {
        const State::ProjGraph &p = s.proj[i];
        if (p.U == U && p.E == s.E && p.G == s.G && p.max_steps == max_steps) exec = p.exec;
    }
    if (!exec) {
        if (capture_projection(s, max_steps, &exec) != LQ_OK) {
            // no graph (a driver without conditional nodes): the host loop from now on
            s.proj_graph = 0;
            return -1;
        }
        if (s.n_proj == State::kProjGraphs) {
            // drop the oldest
            cudaGraphExecDestroy(s.proj[0].exec);
            for (int i = 1; i < s.n_proj; ++i) s.proj[i - 1] = s.proj[i];
            --s.n_proj;
        }
        s.proj[s.n_proj++] = {U, s.E, s.G, max_steps, exec};
    }
    const int slot = prof_begin(s, LQ_KERNEL_GAUSS_SWEEP);
    const cudaError_t e = cudaGraphLaunch(exec, s.stream);
    prof_end(s, slot, LQ_KERNEL_GAUSS_SWEEP);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch (projection)", __LINE__);
    const bool fused = s.precision != LQ_PRECISION_F64;
    // fused sweeps: 1 + 4k of them leave E and G in the other buffers
    if (fused) {
        std::swap(s.E, s.E_alt);
        std::swap(s.G, s.G_alt);
    }
    LQ_CK(cudaMemcpyAsync(s.h_out, s.d_proj, 2 * sizeof(int), cudaMemcpyDeviceToHost, s.stream));
    LQ_CK(cudaStreamSynchronize(s.stream));
    int ctl[2];
    memcpy(ctl, s.h_out, sizeof(ctl));
    // the slot covers the Gauss law, the sweeps (FP64: a step and a Gauss law each, after the
    // transport tables) and the tests
    if (s.prof && slot >= 0)
        s.prof->cnt[slot] = fused ? 1 + ctl[0] + (ctl[0] + 3) / 4 : 2 + 2 * ctl[0] + (ctl[0] + 3) / 4;
    prof_flush(s);
    if (steps_done) *steps_done = ctl[0];
    if (ctl[1] != LQ_OK) return ctl[1];
    if (s.comp) {
        // the sweeps updated the hi parts only: the projected field is hi + 0
        const size_t half = s.efield_bytes() / 2;
        LQ_CK(cudaMemsetAsync((char *)s.E + half, 0, half, s.stream));
    }
    return LQ_OK;
}

// EField::project_to_gauss (src/field.rs:1265-1294): one step, then blocks of four steps
// until the residual of the current field is <= eps * V * 320.  Each sweep also produces
// G and the residual of its result, so the checks after steps 1, 5, 9, ... read it directly.
int project_gauss(State &s, int max_steps, int *steps_done) {
    // FP32 arithmetic: one fused sweep per step (U read once).  FP64: the step and the Gauss
    // law as two kernels, since the sweep's recomputed neighbour updates cost FP64 flops.
    const bool fused = s.precision != LQ_PRECISION_F64;
    if (s.proj_graph) {
        const int rc = project_gauss_graph(s, max_steps, steps_done);
        if (rc != -1) return rc;
    }
    const double threshold = projection_threshold(s);
    const void *U = s.U[s.cur];
    uint32_t n = 0;
    int steps = 0;
    if (fused) {
        LQ_LAUNCH(s, LQ_KERNEL_GAUSS, s.ops->gauss(s, U, &n));
    } else {
        // FP64: the links' transport tables once, then every transport as a real 9x9 product
        LQ_LAUNCH(s, LQ_KERNEL_OTHER, s.ops->adjoint_links(s, U));
        LQ_LAUNCH(s, LQ_KERNEL_GAUSS, s.ops->gauss_adj(s, &n));
    }
    for (;;) {
        if (fused) {
            LQ_LAUNCH(s, LQ_KERNEL_GAUSS_SWEEP, s.ops->gauss_sweep(s, U, &n));
            std::swap(s.E, s.E_alt);
            std::swap(s.G, s.G_alt);
        } else {
            LQ_LAUNCH(s, LQ_KERNEL_GAUSS_SWEEP, s.ops->gauss_step_adj(s));
            LQ_LAUNCH(s, LQ_KERNEL_GAUSS, s.ops->gauss_adj(s, &n));
        }
        ++steps;
        if ((steps - 1) % 4 != 0) continue;
        LQ_LAUNCH(s, LQ_KERNEL_REDUCE, s.ops->finalize(s, 1, n, 0));
        const int rc = fetch_out(s, 1);
        if (rc) return rc;
        const double val_dif = s.h_out[0];
        if (std::isnan(val_dif)) {
            if (steps_done) *steps_done = steps;
            return LQ_ERR_GAUSS_PROJECTION;
        }
        if (val_dif <= threshold) break;
        if (max_steps > 0 && steps + 4 > max_steps) {
            if (steps_done) *steps_done = steps;
            return LQ_ERR_NOT_CONVERGED;
        }
    }
    if (fused && s.comp) {
        // the sweeps updated the hi parts only: the projected field is hi + 0
        const size_t half = s.efield_bytes() / 2;
        LQ_CK(cudaMemsetAsync((char *)s.E + half, 0, half, s.stream));
    }
    if (steps_done) *steps_done = steps;
    return LQ_OK;
}

bool valid_std_dev(double sd) { return sd >= 0.0 && !std::isinf(sd); }

} // namespace

namespace lq {
// lets other translation units of the library report an error through lq_last_error_string
void set_last_error(const char *text) { g_last_error = text; }
} // namespace lq

extern "C" {

int lq_version(void) { return 100; }

const char *lq_last_error_string(void) { return g_last_error.c_str(); }

const char *lq_status_string(int status) {
    switch (status) {
    case LQ_OK: return "ok";
    case LQ_ERR_NON_POSITIVE_SIZE: return "lattice size must be positive and finite";
    case LQ_ERR_DIM_TOO_SMALL: return "number of points per direction must be >= 2";
    case LQ_ERR_ZERO_DIMENSION: return "dimension must be non zero";
    case LQ_ERR_UNSUPPORTED_DIM: return "dimension must be 2, 3 or 4";
    case LQ_ERR_INVALID_NORMAL: return "normal distribution N(0, 0.5/beta) is invalid";
    case LQ_ERR_INCOMPATIBLE_SIZE: return "size of lattice and data are incompatible";
    case LQ_ERR_GAUSS_PROJECTION: return "gauss projection could not finish";
    case LQ_ERR_ZERO_INTEGRATION: return "no integration steps";
    case LQ_ERR_INVALID_ARGUMENT: return "invalid argument";
    case LQ_ERR_NOT_CONVERGED: return "gauss projection reached its step limit";
    case LQ_ERR_WRONG_STATE_KIND: return "integration mode does not match the synchronous/leap-frog kind of the state";
    case LQ_ERR_NO_PENDING: return "no pending HMC proposal";
    case LQ_ERR_CUDA: return "CUDA error";
    case LQ_ERR_OUT_OF_MEMORY: return "device out of memory";
    case LQ_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

int lq_state_create(int dim, int L, double size, double beta, int precision, lq_state **out) {
    if (!out) return LQ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    // LatticeCyclic::new, src/lattice.rs:190-201
    if (dim == 0) return LQ_ERR_ZERO_DIMENSION;
    if (size <= 0.0 || std::isnan(size) || std::isinf(size)) return LQ_ERR_NON_POSITIVE_SIZE;
    if (L < 2) return LQ_ERR_DIM_TOO_SMALL;
    if (dim < 2 || dim > 4) return LQ_ERR_UNSUPPORTED_DIM;
    if (precision != LQ_PRECISION_F64 && precision != LQ_PRECISION_MIXED && precision != LQ_PRECISION_F32)
        return LQ_ERR_INVALID_ARGUMENT;
    uint64_t V = 1;
    for (int i = 0; i < dim; ++i) {
        V *= (uint64_t)L;
        if (V > (1ull << 28)) return LQ_ERR_INVALID_ARGUMENT; // beyond 32-bit link indexing
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        (void)cudaGetLastError();
        g_last_error = "no CUDA device visible";
        return LQ_ERR_NO_DEVICE;
    }
    lq_state *s = new (std::nothrow) lq_state();
    if (!s) return LQ_ERR_OUT_OF_MEMORY;
    s->dim = dim;
    s->L = L;
    s->V = (uint32_t)V;
    s->size = size;
    s->beta = beta;
    s->precision = precision;
    s->real_bytes = precision == LQ_PRECISION_F64 ? 8 : 4;
    s->comp = precision == LQ_PRECISION_MIXED ? 1 : 0;
    s->ops = precision == LQ_PRECISION_F64 ? lq::ops_f64(dim)
             : precision == LQ_PRECISION_MIXED ? lq::ops_mixed(dim)
                                               : lq::ops_f32(dim);
    // strips keep a neighbour along the slowest direction within LQ_BLOCK_REUSE_SITES sites of work,
    // under half of what the resident blocks of the stencil kernels cover at once (152 SMs x 4 blocks
    // x 128 sites)
    s->block_order = lq::make_block_order(dim, (uint32_t)L, 128, LQ_BLOCK_REUSE_SITES);
    s->partial_slots = lq::partial_slots_for(s->V);
    if (s->partial_slots < 1024) s->partial_slots = 1024;
    int rc = LQ_OK;
    auto alloc = [&](void **p, size_t bytes, int line) {
        if (rc) return;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc", line);
    };
    for (int i = 0; i < 3; ++i) alloc(&s->U[i], s->link_bytes(), __LINE__);
    alloc(&s->E, s->efield_bytes(), __LINE__);
    alloc(&s->E_alt, s->efield_bytes(), __LINE__);
    alloc(&s->G, s->gauss_bytes(), __LINE__);
    alloc(&s->G_alt, s->gauss_bytes(), __LINE__);
    if (precision == LQ_PRECISION_F64) alloc(&s->R, s->adjoint_bytes(), __LINE__);
    alloc((void **)&s->partial, sizeof(double) * lq::kPartialRows * (size_t)s->partial_slots, __LINE__);
    alloc((void **)&s->d_out, sizeof(double) * 16, __LINE__);
    if (!rc) {
        cudaError_t e = cudaMallocHost((void **)&s->h_out, sizeof(double) * 16);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMallocHost", __LINE__);
    }
    if (!rc) {
        // every buffer starts zeroed: the padding of the last tile stays zero for the sums
        cudaError_t e = cudaSuccess;
        for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaMemsetAsync(s->U[i], 0, s->link_bytes(), s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->E_alt, 0, s->efield_bytes(), s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->G, 0, s->gauss_bytes(), s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->G_alt, 0, s->gauss_bytes(), s->stream);
        if (e == cudaSuccess) e = s->ops->links_cold(*s, s->U[0]);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->E, 0, s->efield_bytes(), s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "state initialisation", __LINE__);
    }
    if (rc) {
        free_state(s);
        return rc;
    }
    *out = s;
    return LQ_OK;
}

int lq_state_destroy(lq_state *s) {
    if (!s) return LQ_OK;
    cudaStreamSynchronize(s->stream);
    free_state(s);
    return LQ_OK;
}

int lq_state_clone(const lq_state *src, lq_state **out) {
    if (!src || !out) return LQ_ERR_INVALID_ARGUMENT;
    lq_state *c = nullptr;
    int rc = lq_state_create(src->dim, src->L, src->size, src->beta, src->precision, &c);
    if (rc) return rc;
    c->stream = src->stream;
    cudaError_t e = cudaMemcpyAsync(c->U[0], src->U[src->cur], src->link_bytes(), cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->E, src->E, src->efield_bytes(), cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "clone copy", __LINE__);
        free_state(c);
        return rc;
    }
    c->t = src->t;
    c->leap = src->leap;
    c->link_update = src->link_update;
    c->proj_graph = src->proj_graph;
    c->hu_valid = src->hu_valid;
    c->hu = src->hu;
    *out = c;
    return LQ_OK;
}

// ---- whole-state checkpoint: a little-endian header, then the raw device fields
namespace {
constexpr char kCheckpointMagic[8] = {'L', 'Q', 'G', 'P', 'U', 'C', 'K', '1'};
constexpr uint32_t kCheckpointVersion = 1;
struct CheckpointHeader {
    char magic[8];
    uint32_t version;
    int32_t dim, L, precision;
    double size, beta;
    int64_t t;
    int32_t leap, link_update, proj_graph, reserved0;
    uint64_t link_bytes, efield_bytes;
    uint64_t reserved[4];
};
static_assert(sizeof(CheckpointHeader) == 112, "checkpoint header layout");
} // namespace

int lq_state_checkpoint_bytes(const lq_state *s, size_t *bytes) {
    LQ_CHECK_STATE(s);
    if (!bytes) return LQ_ERR_INVALID_ARGUMENT;
    *bytes = sizeof(CheckpointHeader) + s->link_bytes() + s->efield_bytes();
    return LQ_OK;
}

int lq_state_save(lq_state *s, void *buf, size_t n_bytes) {
    LQ_CHECK_STATE(s);
    if (!buf) return LQ_ERR_INVALID_ARGUMENT;
    if (n_bytes != sizeof(CheckpointHeader) + s->link_bytes() + s->efield_bytes()) return LQ_ERR_INCOMPATIBLE_SIZE;
    if (s->has_pending) {
        g_last_error = "lq_state_save: an HMC proposal is pending (lq_hmc_decide first)";
        return LQ_ERR_INVALID_ARGUMENT;
    }
    CheckpointHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kCheckpointMagic, sizeof(h.magic));
    h.version = kCheckpointVersion;
    h.dim = s->dim;
    h.L = s->L;
    h.precision = s->precision;
    h.size = s->size;
    h.beta = s->beta;
    h.t = s->t;
    h.leap = s->leap;
    h.link_update = s->link_update;
    h.proj_graph = s->proj_graph;
    h.link_bytes = s->link_bytes();
    h.efield_bytes = s->efield_bytes();
    char *dst = static_cast<char *>(buf);
    memcpy(dst, &h, sizeof(h));
    LQ_CK(cudaMemcpyAsync(dst + sizeof(h), s->U[s->cur], h.link_bytes, cudaMemcpyDeviceToHost, s->stream));
    LQ_CK(cudaMemcpyAsync(dst + sizeof(h) + h.link_bytes, s->E, h.efield_bytes, cudaMemcpyDeviceToHost, s->stream));
    LQ_CK(sync_stream(*s));
    return LQ_OK;
}

int lq_state_load(const void *buf, size_t n_bytes, lq_state **out) {
    if (!buf || !out) return LQ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    CheckpointHeader h;
    if (n_bytes < sizeof(h)) return LQ_ERR_INCOMPATIBLE_SIZE;
    memcpy(&h, buf, sizeof(h));
    if (memcmp(h.magic, kCheckpointMagic, sizeof(h.magic)) != 0 || h.version != kCheckpointVersion) {
        g_last_error = "lq_state_load: not a checkpoint of this library (magic or version)";
        return LQ_ERR_INVALID_ARGUMENT;
    }
    if (n_bytes != sizeof(h) + h.link_bytes + h.efield_bytes) return LQ_ERR_INCOMPATIBLE_SIZE;
    if (h.leap != 0 && h.leap != 1) return LQ_ERR_INVALID_ARGUMENT;
    if (h.link_update < LQ_LINK_UPDATE_EULER || h.link_update > LQ_LINK_UPDATE_EXP_REUNITARIZE)
        return LQ_ERR_INVALID_ARGUMENT;
    lq_state *s = nullptr;
    int rc = lq_state_create(h.dim, h.L, h.size, h.beta, h.precision, &s);
    if (rc) return rc;
    if (s->link_bytes() != h.link_bytes || s->efield_bytes() != h.efield_bytes) {
        free_state(s);
        return LQ_ERR_INCOMPATIBLE_SIZE;
    }
    const char *src = static_cast<const char *>(buf) + sizeof(h);
    cudaError_t e = cudaMemcpyAsync(s->U[0], src, h.link_bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->E, src + h.link_bytes, h.efield_bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "checkpoint load", __LINE__);
        free_state(s);
        return rc;
    }
    s->cur = 0;
    s->t = h.t;
    s->leap = h.leap;
    s->link_update = h.link_update;
    s->proj_graph = h.proj_graph ? 1 : 0;
    *out = s;
    return LQ_OK;
}

int lq_state_set_projection_graph(lq_state *s, int enable) {
    LQ_CHECK_STATE(s);
    s->proj_graph = enable ? 1 : 0;
    return LQ_OK;
}

int lq_state_set_stream(lq_state *s, void *stream) {
    LQ_CHECK_STATE(s);
    LQ_CK(sync_stream(*s));
    s->stream = (cudaStream_t)stream;
    return LQ_OK;
}

int lq_state_info(const lq_state *s, int *dim, int *L, double *size, double *beta, int *precision,
                  long long *n_sites, long long *t, int *is_leap) {
    LQ_CHECK_STATE(s);
    if (dim) *dim = s->dim;
    if (L) *L = s->L;
    if (size) *size = s->size;
    if (beta) *beta = s->beta;
    if (precision) *precision = s->precision;
    if (n_sites) *n_sites = (long long)s->V;
    if (t) *t = s->t;
    if (is_leap) *is_leap = s->leap;
    return LQ_OK;
}

int lq_state_set_beta(lq_state *s, double beta) {
    LQ_CHECK_STATE(s);
    s->beta = beta;
    s->hu_valid = 0;
    s->has_pending = 0;
    return LQ_OK;
}

int lq_state_set_link_update(lq_state *s, int link_update) {
    LQ_CHECK_STATE(s);
    if (link_update < LQ_LINK_UPDATE_EULER || link_update > LQ_LINK_UPDATE_EXP_REUNITARIZE)
        return LQ_ERR_INVALID_ARGUMENT;
    s->link_update = link_update;
    s->has_pending = 0;
    return LQ_OK;
}

int lq_state_device_bytes(const lq_state *s, size_t *bytes) {
    LQ_CHECK_STATE(s);
    if (!bytes) return LQ_ERR_INVALID_ARGUMENT;
    *bytes = 3 * s->link_bytes() + 2 * s->efield_bytes() + 2 * s->gauss_bytes() +
             sizeof(double) * (lq::kPartialRows * (size_t)s->partial_slots + 16) + s->staging_bytes +
             (s->R ? s->adjoint_bytes() : 0);
    return LQ_OK;
}

// ------------------------------------------------------------------ fields
int lq_links_upload(lq_state *s, const double *links, size_t n) {
    LQ_CHECK_STATE(s);
    if (!links) return LQ_ERR_INVALID_ARGUMENT;
    if (n != (size_t)s->V * s->dim * 18) return LQ_ERR_INCOMPATIBLE_SIZE;
    const size_t bytes = n * sizeof(double);
    int rc = ensure_staging(*s, bytes);
    if (rc) return rc;
    LQ_CK(cudaMemcpyAsync(s->staging, links, bytes, cudaMemcpyHostToDevice, s->stream));
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->links_from_aos(*s, (const double *)s->staging, s->U[s->cur]));
    LQ_CK(sync_stream(*s));
    state_changed(*s);
    return LQ_OK;
}

int lq_links_download(lq_state *s, double *links, size_t n) {
    LQ_CHECK_STATE(s);
    if (!links) return LQ_ERR_INVALID_ARGUMENT;
    if (n != (size_t)s->V * s->dim * 18) return LQ_ERR_INCOMPATIBLE_SIZE;
    const size_t bytes = n * sizeof(double);
    int rc = ensure_staging(*s, bytes);
    if (rc) return rc;
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->links_to_aos(*s, s->U[s->cur], (double *)s->staging));
    LQ_CK(cudaMemcpyAsync(links, s->staging, bytes, cudaMemcpyDeviceToHost, s->stream));
    LQ_CK(sync_stream(*s));
    return LQ_OK;
}

int lq_links_set_cold(lq_state *s) {
    LQ_CHECK_STATE(s);
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->links_cold(*s, s->U[s->cur]));
    LQ_CK(sync_stream(*s));
    state_changed(*s);
    return LQ_OK;
}

int lq_links_random(lq_state *s, uint64_t seed) {
    LQ_CHECK_STATE(s);
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->links_random(*s, s->U[s->cur], seed));
    LQ_CK(sync_stream(*s));
    state_changed(*s);
    return LQ_OK;
}

int lq_efield_upload(lq_state *s, const double *efield, size_t n) {
    LQ_CHECK_STATE(s);
    if (!efield) return LQ_ERR_INVALID_ARGUMENT;
    if (n != (size_t)s->V * s->dim * 8) return LQ_ERR_INCOMPATIBLE_SIZE;
    const size_t bytes = n * sizeof(double);
    int rc = ensure_staging(*s, bytes);
    if (rc) return rc;
    LQ_CK(cudaMemcpyAsync(s->staging, efield, bytes, cudaMemcpyHostToDevice, s->stream));
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->efield_from_aos(*s, (const double *)s->staging));
    LQ_CK(sync_stream(*s));
    s->has_pending = 0;
    return LQ_OK;
}

int lq_efield_download(lq_state *s, double *efield, size_t n) {
    LQ_CHECK_STATE(s);
    if (!efield) return LQ_ERR_INVALID_ARGUMENT;
    if (n != (size_t)s->V * s->dim * 8) return LQ_ERR_INCOMPATIBLE_SIZE;
    const size_t bytes = n * sizeof(double);
    int rc = ensure_staging(*s, bytes);
    if (rc) return rc;
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->efield_to_aos(*s, s->E, (double *)s->staging));
    LQ_CK(cudaMemcpyAsync(efield, s->staging, bytes, cudaMemcpyDeviceToHost, s->stream));
    LQ_CK(sync_stream(*s));
    return LQ_OK;
}

int lq_efield_set_cold(lq_state *s) {
    LQ_CHECK_STATE(s);
    LQ_CK(cudaMemsetAsync(s->E, 0, s->efield_bytes(), s->stream));
    LQ_CK(sync_stream(*s));
    s->has_pending = 0;
    return LQ_OK;
}

int lq_efield_random_normal(lq_state *s, uint64_t seed, uint64_t counter, double std_dev) {
    LQ_CHECK_STATE(s);
    if (!valid_std_dev(std_dev)) return LQ_ERR_INVALID_NORMAL;
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->efield_normal(*s, seed, counter, std_dev));
    LQ_CK(sync_stream(*s));
    s->has_pending = 0;
    return LQ_OK;
}

// ------------------------------------------------------------------ observables
int lq_hamiltonian_links(lq_state *s, double *out) {
    LQ_CHECK_STATE(s);
    if (!out) return LQ_ERR_INVALID_ARGUMENT;
    if (!s->hu_valid) {
        int rc = plaquette_sums(*s, s->U[s->cur], 0);
        if (!rc) rc = fetch_out(*s, 3);
        if (rc) return rc;
        s->hu = s->h_out[0] * s->beta;
        s->hu_valid = 1;
    }
    *out = s->hu;
    return LQ_OK;
}

int lq_hamiltonian_efield(lq_state *s, double *out) {
    LQ_CHECK_STATE(s);
    if (!out) return LQ_ERR_INVALID_ARGUMENT;
    int rc = efield_sumsq(*s, 0);
    if (!rc) rc = fetch_out(*s, 1);
    if (rc) return rc;
    *out = s->h_out[0] / 2.0 * s->beta;
    return LQ_OK;
}

int lq_hamiltonian_total(lq_state *s, double *out) {
    LQ_CHECK_STATE(s);
    if (!out) return LQ_ERR_INVALID_ARGUMENT;
    double hu = 0.0, he = 0.0;
    int rc = lq_hamiltonian_links(s, &hu);
    if (!rc) rc = lq_hamiltonian_efield(s, &he);
    if (rc) return rc;
    *out = hu + he;
    return LQ_OK;
}

int lq_average_trace_plaquette(lq_state *s, double *re, double *im) {
    LQ_CHECK_STATE(s);
    int rc = plaquette_sums(*s, s->U[s->cur], 0);
    if (!rc) rc = fetch_out(*s, 3);
    if (rc) return rc;
    const double n_plaq = (double)((uint64_t)s->V * (uint64_t)((s->dim * (s->dim - 1)) / 2));
    if (re) *re = s->h_out[1] / n_plaq;
    if (im) *im = s->h_out[2] / n_plaq;
    s->hu = s->h_out[0] * s->beta;
    s->hu_valid = 1;
    return LQ_OK;
}

int lq_gauss_sum_div(lq_state *s, double *out) {
    LQ_CHECK_STATE(s);
    if (!out) return LQ_ERR_INVALID_ARGUMENT;
    uint32_t n = 0;
    LQ_LAUNCH(*s, LQ_KERNEL_GAUSS, s->ops->gauss(*s, s->U[s->cur], &n));
    LQ_LAUNCH(*s, LQ_KERNEL_REDUCE, s->ops->finalize(*s, 1, n, 0));
    int rc = fetch_out(*s, 1);
    if (rc) return rc;
    *out = s->h_out[0];
    return LQ_OK;
}

int lq_gauss_download(lq_state *s, double *out, size_t n_doubles) {
    LQ_CHECK_STATE(s);
    if (!out) return LQ_ERR_INVALID_ARGUMENT;
    if (n_doubles != (size_t)s->V * 8) return LQ_ERR_INCOMPATIBLE_SIZE;
    const size_t bytes = n_doubles * sizeof(double);
    int rc = ensure_staging(*s, bytes);
    if (rc) return rc;
    uint32_t n = 0;
    LQ_LAUNCH(*s, LQ_KERNEL_GAUSS, s->ops->gauss(*s, s->U[s->cur], &n));
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->gauss_to_aos(*s, (double *)s->staging));
    LQ_CK(cudaMemcpyAsync(out, s->staging, bytes, cudaMemcpyDeviceToHost, s->stream));
    LQ_CK(sync_stream(*s));
    return LQ_OK;
}

// ------------------------------------------------------------------ clover observables
namespace {
int clover_download(lq_state *s, double *out, size_t n, bool magnetic) {
    LQ_CHECK_STATE(s);
    if (!out) return LQ_ERR_INVALID_ARGUMENT;
    const size_t per_site = magnetic ? (size_t)s->dim : (size_t)(s->dim * (s->dim - 1) / 2);
    if (n != (size_t)s->V * per_site * 18) return LQ_ERR_INCOMPATIBLE_SIZE;
    int rc = ensure_staging(*s, n * sizeof(double));
    if (rc) return rc;
    double *d = (double *)s->staging;
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->clover_fields(*s, s->U[s->cur], magnetic ? nullptr : d, magnetic ? d : nullptr));
    LQ_CK(cudaMemcpyAsync(out, d, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    LQ_CK(sync_stream(*s));
    return LQ_OK;
}
} // namespace

int lq_field_strength(lq_state *s, double *out, size_t n_doubles) { return clover_download(s, out, n_doubles, false); }
int lq_magnetic_field(lq_state *s, double *out, size_t n_doubles) { return clover_download(s, out, n_doubles, true); }

// ------------------------------------------------------------------ local Monte Carlo sweeps
namespace {
int mc_sweep(lq_state *s, int alg, int n_update, double spread, uint64_t seed, uint64_t sweep,
             long long *n_accepted, double *prob_mean) {
    LQ_CHECK_STATE(s);
    if (s->L % 2 != 0) {
        lq::set_last_error("checkerboard sweeps need an even number of points per direction");
        return LQ_ERR_INVALID_ARGUMENT;
    }
    if (s->leap) return LQ_ERR_WRONG_STATE_KIND;
    State &st = *s;
    state_changed(st);
    double acc = 0.0, psum = 0.0;
    for (int mu = 0; mu < st.dim; ++mu)
        for (int parity = 0; parity < 2; ++parity) {
            uint32_t n = 0;
            LQ_LAUNCH(st, LQ_KERNEL_OTHER,
                      st.ops->mc_sweep(st, st.U[st.cur], alg, mu, parity, st.beta, seed, sweep, n_update, spread, &n));
            if (alg == lq::MC_METROPOLIS) {
                // rows 0 (accepted) and 1 (probabilities) of the partials; the third row is unused
                LQ_LAUNCH(st, LQ_KERNEL_REDUCE, st.ops->finalize(st, 3, n, 0));
                const int rc = fetch_out(st, 2);
                if (rc) return rc;
                acc += st.h_out[0];
                psum += st.h_out[1];
            }
        }
    LQ_CK(sync_stream(st));
    const double n_links = (double)st.V * st.dim;
    if (n_accepted) *n_accepted = (long long)acc;
    if (prob_mean) *prob_mean = psum / n_links;
    return LQ_OK;
}
} // namespace

int lq_metropolis_sweep(lq_state *s, int n_update, double spread, uint64_t seed, uint64_t sweep,
                        long long *n_accepted, double *prob_mean) {
    LQ_CHECK_STATE(s);
    // MetropolisHastingsSweep::new (metropolis_hastings_sweep.rs:86-97)
    if (n_update <= 0 || !(spread > 0.0) || !(spread < 1.0)) return LQ_ERR_INVALID_ARGUMENT;
    return mc_sweep(s, lq::MC_METROPOLIS, n_update, spread, seed, sweep, n_accepted, prob_mean);
}

int lq_heat_bath_sweep(lq_state *s, uint64_t seed, uint64_t sweep) {
    LQ_CHECK_STATE(s);
    if (!(s->beta > 0.0) || std::isinf(s->beta)) return LQ_ERR_INVALID_ARGUMENT;
    return mc_sweep(s, lq::MC_HEAT_BATH, 1, 0.5, seed, sweep, nullptr, nullptr);
}

int lq_overrelaxation_sweep(lq_state *s, int method) {
    LQ_CHECK_STATE(s);
    if (method != LQ_OVERRELAX_ROTATION && method != LQ_OVERRELAX_REVERSE) return LQ_ERR_INVALID_ARGUMENT;
    const int alg = method == LQ_OVERRELAX_ROTATION ? lq::MC_OVERRELAX_ROTATION : lq::MC_OVERRELAX_REVERSE;
    return mc_sweep(s, alg, 1, 0.5, 0, 0, nullptr, nullptr);
}

// ------------------------------------------------------------------ differentiation
int lq_wilson_action(lq_state *s, double *out) { return lq_hamiltonian_links(s, out); }

int lq_wilson_action_backward(lq_state *s, double *grad, size_t n) {
    LQ_CHECK_STATE(s);
    if (!grad) return LQ_ERR_INVALID_ARGUMENT;
    if (n != (size_t)s->V * s->dim * 8) return LQ_ERR_INCOMPATIBLE_SIZE;
    const size_t bytes = n * sizeof(double);
    int rc = ensure_staging(*s, bytes);
    if (rc) return rc;
    s->has_pending = 0;
    // dS/dtheta^a = beta/3 Im Tr(T^a U Sigma): S = beta sum (1 - Re Tr P / 3) and
    // d/dtheta Re Tr(exp(i theta T) U Sigma) = -Im Tr(T U Sigma) at theta = 0
    LQ_CK(cudaMemsetAsync(s->E_alt, 0, s->efield_bytes(), s->stream));
    LQ_LAUNCH(*s, LQ_KERNEL_MD, s->ops->force(*s, s->U[s->cur], s->E_alt, s->beta / 3.0));
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->efield_to_aos(*s, s->E_alt, (double *)s->staging));
    LQ_CK(cudaMemcpyAsync(grad, s->staging, bytes, cudaMemcpyDeviceToHost, s->stream));
    LQ_CK(sync_stream(*s));
    return LQ_OK;
}

int lq_link_rotate(lq_state *s, long long link, int generator, double angle) {
    LQ_CHECK_STATE(s);
    if (link < 0 || link >= (long long)s->V * s->dim || generator < 0 || generator > 7) return LQ_ERR_INVALID_ARGUMENT;
    const uint32_t site = (uint32_t)(link / s->dim);
    const int mu = (int)(link % s->dim);
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->link_rotate(*s, s->U[s->cur], site, mu, generator, angle));
    LQ_CK(sync_stream(*s));
    state_changed(*s);
    return LQ_OK;
}

// Reverse-mode adjoint of n symplectic leap-frog steps for O = Re average_trace_plaquette / 3
// of the final links.  Pass 1 runs the steps forward from (U0, E0), keeping the state that
// enters every c-th step; the reverse pass then takes the segments from last to first,
// recomputes the segment's links U_k and kicked momenta E_k from its checkpoint, and applies
// the adjoint of each drift and kick (adjoint.cuh).  Device memory: ceil(n/c) checkpoints +
// c+1 links and c momenta of one segment + the two cotangents; c = ceil(sqrt(n)) by default.
int lq_leapfrog_adjoint(lq_state *s, double dt, int n_steps, int checkpoint_every, double *objective,
                        double *d_objective_d_beta, double *grad_links, size_t n_link_doubles, double *grad_efield,
                        size_t n_efield_doubles, size_t *work_bytes) {
    LQ_CHECK_STATE(s);
    if (n_steps <= 0) return LQ_ERR_ZERO_INTEGRATION;
    if (s->leap) return LQ_ERR_WRONG_STATE_KIND;
    if (!std::isfinite(dt) || checkpoint_every < 0) return LQ_ERR_INVALID_ARGUMENT;
    if (grad_links && n_link_doubles != (size_t)s->V * s->dim * 18) return LQ_ERR_INCOMPATIBLE_SIZE;
    if (grad_efield && n_efield_doubles != (size_t)s->V * s->dim * 8) return LQ_ERR_INCOMPATIBLE_SIZE;
    State &st = *s;
    const int n = n_steps;
    int c = checkpoint_every > 0 ? checkpoint_every : (int)std::ceil(std::sqrt((double)n));
    if (c > n) c = n;
    const int n_ck = (n + c - 1) / c;
    const size_t ub = st.link_bytes(), eb = st.efield_bytes();
    const size_t cu_bytes = st.link_elems() * 2 * st.real_bytes, ce_bytes = st.efield_elems() * st.real_bytes;
    const size_t total = (size_t)n_ck * (ub + eb) + (size_t)(c + 1) * ub + (size_t)c * eb + cu_bytes + ce_bytes;
    if (work_bytes) *work_bytes = total;
    char *arena = nullptr;
    LQ_CK(cudaMalloc((void **)&arena, total));
    auto ck_u = [&](int i) { return arena + (size_t)i * (ub + eb); };
    auto ck_e = [&](int i) { return arena + (size_t)i * (ub + eb) + ub; };
    char *seg = arena + (size_t)n_ck * (ub + eb);
    auto seg_u = [&](int j) { return seg + (size_t)j * ub; };
    auto seg_e = [&](int j) { return seg + (size_t)(c + 1) * ub + (size_t)j * eb; };
    void *lam_u = seg + (size_t)(c + 1) * ub + (size_t)c * eb;
    void *lam_e = (char *)lam_u + cu_bytes;
    const int KD = lq::MD_KICK | lq::MD_DRIFT;
    const double ce = -std::sqrt(2.0 / 3.0) / st.size; // force coefficient
    const double kappa = std::sqrt(2.0 * 3.0) / st.size * dt;
    const double n_plaq = (double)((uint64_t)st.V * (uint64_t)((st.dim * (st.dim - 1)) / 2));
    int rc = LQ_OK;
    auto run = [&]() -> int {
        // pass 1: forward, keeping the state that enters steps 0, c, 2c, ...
        LQ_CK(cudaMemcpyAsync(seg_u(0), st.U[st.cur], ub, cudaMemcpyDeviceToDevice, st.stream));
        LQ_CK(cudaMemcpyAsync(seg_e(0), st.E, eb, cudaMemcpyDeviceToDevice, st.stream));
        int a = 0;
        for (int k = 0; k < n; ++k) {
            if (k % c == 0) {
                LQ_CK(cudaMemcpyAsync(ck_u(k / c), seg_u(a), ub, cudaMemcpyDeviceToDevice, st.stream));
                LQ_CK(cudaMemcpyAsync(ck_e(k / c), seg_e(0), eb, cudaMemcpyDeviceToDevice, st.stream));
            }
            LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, seg_u(a), seg_u(1 - a), seg_e(0), seg_e(0), KD,
                                                  k == 0 ? 0.0 : dt / 2.0, dt / 2.0, dt));
            a = 1 - a;
        }
        int r = plaquette_sums(st, seg_u(a), 0);
        if (!r) r = fetch_out(st, 3);
        if (r) return r;
        if (objective) *objective = st.h_out[1] / n_plaq / 3.0;
        // cotangents at the end: lam_U = dO/dU_n, lam_E = 0 (O does not depend on E_n)
        LQ_LAUNCH(st, LQ_KERNEL_OTHER, st.ops->adj_init(st, seg_u(a), lam_u, 1.0 / (3.0 * n_plaq)));
        LQ_CK(cudaMemsetAsync(lam_e, 0, ce_bytes, st.stream));
        for (int sgm = n_ck - 1; sgm >= 0; --sgm) {
            const int k0 = sgm * c, len = std::min(c, n - k0);
            // recompute the segment: seg_u(j) = U_{k0+j}, seg_e(j) = momenta after kick k0+j
            LQ_CK(cudaMemcpyAsync(seg_u(0), ck_u(sgm), ub, cudaMemcpyDeviceToDevice, st.stream));
            for (int j = 0; j < len; ++j) {
                const int k = k0 + j;
                LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, seg_u(j), seg_u(j + 1), j == 0 ? ck_e(sgm) : seg_e(j - 1),
                                                      seg_e(j), KD, k == 0 ? 0.0 : dt / 2.0, dt / 2.0, dt));
            }
            for (int j = len - 1; j >= 0; --j) {
                const int k = k0 + j;
                LQ_LAUNCH(st, LQ_KERNEL_OTHER, st.ops->adj_drift(st, seg_u(j), seg_e(j), lam_u, lam_e, kappa));
                const double h = k == 0 ? dt / 2.0 : dt;
                LQ_LAUNCH(st, LQ_KERNEL_OTHER, st.ops->adj_kick(st, seg_u(j), lam_e, lam_u, h * ce));
            }
        }
        // dO/dbeta for E0(beta) = E0 beta0 / beta: -(1/beta) sum_l,a lam_E^a e0^a
        uint32_t np = 0;
        LQ_LAUNCH(st, LQ_KERNEL_REDUCE, st.ops->dot(st, lam_e, st.E, &np));
        LQ_LAUNCH(st, LQ_KERNEL_REDUCE, st.ops->finalize(st, 1, np, 0));
        r = fetch_out(st, 1);
        if (r) return r;
        if (d_objective_d_beta) *d_objective_d_beta = -st.h_out[0] / st.beta;
        if (grad_links) {
            r = ensure_staging(st, n_link_doubles * sizeof(double));
            if (r) return r;
            LQ_LAUNCH(st, LQ_KERNEL_OTHER, st.ops->cot_links_to_aos(st, lam_u, (double *)st.staging));
            LQ_CK(cudaMemcpyAsync(grad_links, st.staging, n_link_doubles * sizeof(double), cudaMemcpyDeviceToHost,
                                  st.stream));
            LQ_CK(sync_stream(st));
        }
        if (grad_efield) {
            r = ensure_staging(st, n_efield_doubles * sizeof(double));
            if (r) return r;
            LQ_LAUNCH(st, LQ_KERNEL_OTHER, st.ops->cot_efield_to_aos(st, lam_e, (double *)st.staging));
            LQ_CK(cudaMemcpyAsync(grad_efield, st.staging, n_efield_doubles * sizeof(double), cudaMemcpyDeviceToHost,
                                  st.stream));
            LQ_CK(sync_stream(st));
        }
        return LQ_OK;
    };
    rc = run();
    cudaStreamSynchronize(st.stream);
    cudaFree(arena);
    return rc;
}

// ------------------------------------------------------------------ updates
int lq_project_gauss(lq_state *s, int max_steps, int *steps_done) {
    LQ_CHECK_STATE(s);
    s->has_pending = 0;
    return project_gauss(*s, max_steps, steps_done);
}

int lq_normalize_link_matrices(lq_state *s) {
    LQ_CHECK_STATE(s);
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->normalize(*s, s->U[s->cur]));
    LQ_CK(sync_stream(*s));
    state_changed(*s);
    return LQ_OK;
}

int lq_integrate(lq_state *s, int mode, double dt, int n) {
    LQ_CHECK_STATE(s);
    if (mode < LQ_SYNC_SYNC || mode > LQ_SYMPLECTIC_EXP_REUNITARIZE) return LQ_ERR_INVALID_ARGUMENT;
    if (n <= 0) return LQ_ERR_ZERO_INTEGRATION;
    const bool needs_leap = (mode == LQ_LEAP_LEAP || mode == LQ_LEAP_SYNC);
    if ((needs_leap && !s->leap) || (!needs_leap && s->leap)) return LQ_ERR_WRONG_STATE_KIND;
    if ((mode == LQ_SYNC_LEAP || mode == LQ_LEAP_SYNC) && n != 1) return LQ_ERR_WRONG_STATE_KIND;
    State &st = *s;
    state_changed(st);
    const int KD = lq::MD_KICK | lq::MD_DRIFT;
    int a = st.cur, b = other_buffer(st, st.cur, -1);
    switch (mode) {
    case LQ_SYNC_SYNC:
        for (int i = 0; i < n; ++i) {
            LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[a], st.U[b], st.E, st.E, KD | lq::MD_DRIFT_OLD_E, 0.0, dt, dt));
            const int t = a;
            a = b;
            b = t;
        }
        st.cur = a;
        st.t += n;
        break;
    case LQ_SYNC_LEAP:
        LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[a], st.U[a], st.E, st.E, lq::MD_KICK, 0.0, dt / 2.0, 0.0));
        st.leap = 1;
        break;
    case LQ_LEAP_LEAP:
        LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[a], st.U[b], st.E, st.E, lq::MD_DRIFT, 0.0, 0.0, dt));
        for (int i = 1; i < n; ++i) {
            LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[b], st.U[a], st.E, st.E, KD, 0.0, dt, dt));
            const int t = a;
            a = b;
            b = t;
        }
        LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[b], st.U[b], st.E, st.E, lq::MD_KICK, 0.0, dt, 0.0));
        st.cur = b;
        st.t += n;
        break;
    case LQ_LEAP_SYNC:
        LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[a], st.U[b], st.E, st.E, lq::MD_DRIFT, 0.0, 0.0, dt));
        LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[b], st.U[b], st.E, st.E, lq::MD_KICK, 0.0, dt / 2.0, 0.0));
        st.cur = b;
        st.leap = 0;
        st.t += 1;
        break;
    default: { // LQ_SYMPLECTIC, LQ_SYMPLECTIC_EXP, LQ_SYMPLECTIC_EXP_REUNITARIZE
        int fin = -1;
        const int lu = mode == LQ_SYMPLECTIC_EXP ? LQ_LINK_UPDATE_EXP
                       : mode == LQ_SYMPLECTIC_EXP_REUNITARIZE ? LQ_LINK_UPDATE_EXP_REUNITARIZE
                                                               : LQ_LINK_UPDATE_EULER;
        int rc = run_symplectic(st, st.cur, dt, n, false, lu, &fin);
        if (rc) return rc;
        st.cur = fin;
        st.t += n;
        break;
    }
    }
    LQ_CK(sync_stream(st));
    return LQ_OK;
}

int lq_leapfrog_n(lq_state *s, double dt, int n) {
    LQ_CHECK_STATE(s);
    if (n <= 0) return LQ_ERR_ZERO_INTEGRATION;
    if (s->leap) return LQ_ERR_WRONG_STATE_KIND;
    State &st = *s;
    state_changed(st);
    const int KD = lq::MD_KICK | lq::MD_DRIFT;
    int a = st.cur, b = other_buffer(st, st.cur, -1);
    // sync -> leap: E += dt/2 F(U0)
    LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[a], st.U[a], st.E, st.E, lq::MD_KICK, 0.0, dt / 2.0, 0.0));
    // first drift (of leap_leap, or of leap_sync when n == 1)
    LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[a], st.U[b], st.E, st.E, lq::MD_DRIFT, 0.0, 0.0, dt));
    for (int i = 1; i < n; ++i) {
        LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[b], st.U[a], st.E, st.E, KD, 0.0, dt, dt));
        const int t = a;
        a = b;
        b = t;
    }
    // leap -> sync: E += dt/2 F(U_n)
    LQ_LAUNCH(st, LQ_KERNEL_MD, st.ops->md(st, st.U[b], st.U[b], st.E, st.E, lq::MD_KICK, 0.0, dt / 2.0, 0.0));
    st.cur = b;
    st.t += n;
    LQ_CK(sync_stream(st));
    return LQ_OK;
}

// ------------------------------------------------------------------ HMC
int lq_hmc_refresh(lq_state *s, uint64_t seed, uint64_t counter, int max_gauss_steps, int *gauss_steps) {
    LQ_CHECK_STATE(s);
    const double sd = 0.5 / s->beta;
    if (!valid_std_dev(sd)) return LQ_ERR_INVALID_NORMAL;
    s->has_pending = 0;
    s->leap = 0;
    s->t = 0;
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->efield_normal(*s, seed, counter, sd));
    return project_gauss(*s, max_gauss_steps, gauss_steps);
}

int lq_hmc_refresh_upload(lq_state *s, const double *efield_raw, size_t n, int max_gauss_steps, int *gauss_steps) {
    LQ_CHECK_STATE(s);
    if (!valid_std_dev(0.5 / s->beta)) return LQ_ERR_INVALID_NORMAL;
    if (!efield_raw) return LQ_ERR_INVALID_ARGUMENT;
    if (n != (size_t)s->V * s->dim * 8) return LQ_ERR_INCOMPATIBLE_SIZE;
    const size_t bytes = n * sizeof(double);
    int rc = ensure_staging(*s, bytes);
    if (rc) return rc;
    LQ_CK(cudaMemcpyAsync(s->staging, efield_raw, bytes, cudaMemcpyHostToDevice, s->stream));
    // the projection below reads the hi parts and clears the lo parts
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->efield_hi_from_aos(*s, (const double *)s->staging));
    s->has_pending = 0;
    s->leap = 0;
    s->t = 0;
    return project_gauss(*s, max_gauss_steps, gauss_steps);
}

int lq_efield_prefetch(lq_state *s, const double *efield_raw, size_t n) {
    LQ_CHECK_STATE(s);
    if (!efield_raw) return LQ_ERR_INVALID_ARGUMENT;
    if (n != (size_t)s->V * s->dim * 8) return LQ_ERR_INCOMPATIBLE_SIZE;
    const size_t bytes = n * sizeof(double);
    if (!s->copy_stream) {
        LQ_CK(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
        LQ_CK(cudaEventCreateWithFlags(&s->prefetch_done, cudaEventDisableTiming));
        LQ_CK(cudaEventCreateWithFlags(&s->prefetch_free, cudaEventDisableTiming));
        LQ_CK(cudaEventRecord(s->prefetch_free, s->stream));
    }
    if (s->prefetch_bytes < bytes) {
        LQ_CK(cudaStreamSynchronize(s->copy_stream));
        if (s->prefetch) LQ_CK(cudaFree(s->prefetch));
        s->prefetch = nullptr;
        s->prefetch_bytes = 0;
        LQ_CK(cudaMalloc(&s->prefetch, bytes));
        s->prefetch_bytes = bytes;
    }
    // the copy may overwrite the buffer only once its previous contents have been converted
    LQ_CK(cudaStreamWaitEvent(s->copy_stream, s->prefetch_free, 0));
    LQ_CK(cudaMemcpyAsync(s->prefetch, efield_raw, bytes, cudaMemcpyHostToDevice, s->copy_stream));
    LQ_CK(cudaEventRecord(s->prefetch_done, s->copy_stream));
    s->prefetch_pending = 1;
    return LQ_OK;
}

int lq_hmc_refresh_prefetched(lq_state *s, int max_gauss_steps, int *gauss_steps) {
    LQ_CHECK_STATE(s);
    if (!s->prefetch_pending) return LQ_ERR_NO_PENDING;
    if (!valid_std_dev(0.5 / s->beta)) return LQ_ERR_INVALID_NORMAL;
    LQ_CK(cudaStreamWaitEvent(s->stream, s->prefetch_done, 0));
    // the projection below reads the hi parts and clears the lo parts
    LQ_LAUNCH(*s, LQ_KERNEL_OTHER, s->ops->efield_hi_from_aos(*s, (const double *)s->prefetch));
    LQ_CK(cudaEventRecord(s->prefetch_free, s->stream));
    s->prefetch_pending = 0;
    s->has_pending = 0;
    s->leap = 0;
    s->t = 0;
    return project_gauss(*s, max_gauss_steps, gauss_steps);
}

int lq_hmc_propose(lq_state *s, double dt, int n_steps, double *prob, double *h_old, double *h_new) {
    LQ_CHECK_STATE(s);
    if (n_steps <= 0) return LQ_ERR_ZERO_INTEGRATION;
    if (s->leap) return LQ_ERR_WRONG_STATE_KIND;
    State &st = *s;
    st.has_pending = 0;
    int rc = LQ_OK;
    // H of the start state: d_out[0..2] plaquette sums (unless cached); sum e^2 in d_out[3] (FP64,
    // here) or d_out[6] (FP32 arithmetic, from the difference kernel after the MD, which reads the
    // start momenta anyway: they stay in st.E)
    if (!st.hu_valid) {
        rc = plaquette_sums(st, st.U[st.cur], 0);
        if (rc) return rc;
    }
    if (st.precision == LQ_PRECISION_F64) {
        rc = efield_sumsq(st, 3);
        if (rc) return rc;
    }
    int fin = -1;
    rc = run_symplectic(st, st.cur, dt, n_steps, true, st.link_update, &fin); // start momenta stay in st.E
    if (rc) return rc;
    double hu_old = 0.0, he_old = 0.0, hu_new = 0.0, he_new = 0.0;
    if (st.precision == LQ_PRECISION_F64) {
        // probability_of_replacement (hybrid_monte_carlo.rs:584-589): both Hamiltonians summed
        // separately, as the reference does; d_out[4..6], d_out[7]
        std::swap(st.E, st.E_alt);
        rc = plaquette_sums(st, st.U[fin], 4);
        if (!rc) rc = efield_sumsq(st, 7);
        if (!rc) rc = fetch_out(st, 8);
        if (rc) return rc;
        hu_old = st.hu_valid ? st.hu : st.h_out[0] * st.beta;
        he_old = st.h_out[3] / 2.0 * st.beta;
        hu_new = st.h_out[4] * st.beta;
        he_new = st.h_out[7] / 2.0 * st.beta;
    } else {
        // FP32 arithmetic: Delta H from the difference kernels (no cancellation between two
        // large sums); d_out[4] = sum Re Tr[P' - P], d_out[5] = sum (e' - e)(e' + e),
        // d_out[6] = sum e^2 of the start momenta
        uint32_t n = 0;
        LQ_LAUNCH(st, LQ_KERNEL_PLAQUETTE, st.ops->plaquette_delta(st, st.U[st.cur], st.U[fin], &n));
        LQ_LAUNCH(st, LQ_KERNEL_REDUCE, st.ops->finalize(st, 1, n, 4));
        LQ_LAUNCH(st, LQ_KERNEL_REDUCE, st.ops->efield_sumsq_delta(st, st.E, st.E_alt, &n));
        LQ_LAUNCH(st, LQ_KERNEL_REDUCE, st.ops->finalize(st, 2, n, 5));
        rc = fetch_out(st, 7);
        if (rc) return rc;
        std::swap(st.E, st.E_alt);
        hu_old = st.hu_valid ? st.hu : st.h_out[0] * st.beta;
        he_old = st.h_out[6] / 2.0 * st.beta;
        hu_new = hu_old - st.h_out[4] / 3.0 * st.beta;
        he_new = he_old + st.h_out[5] / 2.0 * st.beta;
    }
    const double h0 = hu_old + he_old, h1 = hu_new + he_new;
    const double dh = (st.precision == LQ_PRECISION_F64) ? h1 - h0 : (hu_new - hu_old) + (he_new - he_old);
    // probability_of_replacement, hybrid_monte_carlo.rs:584-589 (NaN clamps to 1 as f64::min does)
    double p = std::fmax(std::fmin(std::exp(-dh), 1.0), 0.0);
    if (prob) *prob = p;
    if (h_old) *h_old = h0;
    if (h_new) *h_new = h1;
    st.hu = hu_old;
    st.hu_valid = 1;
    st.pending_hu_old = hu_old;
    st.pending_hu_new = hu_new;
    st.pending_dh = dh;
    st.pending_buf = fin;
    st.has_pending = 1;
    st.t = n_steps;
    return LQ_OK;
}

int lq_hmc_decide(lq_state *s, int accept) {
    LQ_CHECK_STATE(s);
    if (!s->has_pending) return LQ_ERR_NO_PENDING;
    if (accept) {
        s->cur = s->pending_buf;
        s->hu = s->pending_hu_new;
    } else {
        s->hu = s->pending_hu_old;
    }
    s->hu_valid = 1;
    s->has_pending = 0;
    s->pending_buf = -1;
    return LQ_OK;
}

int lq_hmc_trajectory(lq_state *s, double dt, int n_steps, uint64_t seed, uint64_t counter, double uniform,
                      int max_gauss_steps, int *accepted, double *prob, double *delta_h, int *gauss_steps) {
    LQ_CHECK_STATE(s);
    if (n_steps <= 0) return LQ_ERR_ZERO_INTEGRATION;
    int rc = lq_hmc_refresh(s, seed, counter, max_gauss_steps, gauss_steps);
    if (rc) return rc;
    double p = 0.0, h0 = 0.0, h1 = 0.0;
    rc = lq_hmc_propose(s, dt, n_steps, &p, &h0, &h1);
    if (rc) return rc;
    const int acc = (p >= 1.0 || uniform < p) ? 1 : 0;
    const double dh = s->pending_dh;
    rc = lq_hmc_decide(s, acc);
    if (rc) return rc;
    if (accepted) *accepted = acc;
    if (prob) *prob = p;
    if (delta_h) *delta_h = dh;
    return LQ_OK;
}

int lq_profile_enable(lq_state *s, int on) {
    LQ_CHECK_STATE(s);
    LQ_CK(sync_stream(*s));
    if (on && !s->prof) {
        lq::Prof *p = new (std::nothrow) lq::Prof();
        if (!p) return LQ_ERR_OUT_OF_MEMORY;
        for (int i = 0; i < 2 * lq::kProfPool; ++i) {
            cudaError_t e = cudaEventCreate(&p->ev[i]);
            if (e != cudaSuccess) {
                for (int j = 0; j < i; ++j) cudaEventDestroy(p->ev[j]);
                delete p;
                return cuda_fail(e, "cudaEventCreate", __LINE__);
            }
        }
        s->prof = p;
    } else if (!on) {
        prof_free(*s);
    }
    return LQ_OK;
}

int lq_bounds_check(int *enabled, unsigned long long *violations, unsigned long long *first_bad, int reset) {
    if (enabled) *enabled = LQ_BOUNDS_CHECK;
    unsigned long long n = 0, first = 0;
    for (lq::BoundsReader read : lq::bounds_readers()) {
        const int e = read(&n, &first, reset);
        if (e) return cuda_fail((cudaError_t)e, "reading the index-check counters", __LINE__);
    }
    if (violations) *violations = n;
    if (first_bad) *first_bad = first;
    return LQ_OK;
}

int lq_profile_classes(lq_state *s, unsigned mask) {
    LQ_CHECK_STATE(s);
    s->prof_mask = mask;
    return LQ_OK;
}

int lq_profile_read(lq_state *s, int kernel_class, long long *launches, double *total_ms, int reset) {
    LQ_CHECK_STATE(s);
    if (kernel_class < 0 || kernel_class >= LQ_KERNEL_CLASSES) return LQ_ERR_INVALID_ARGUMENT;
    LQ_CK(sync_stream(*s));
    if (!s->prof) {
        if (launches) *launches = 0;
        if (total_ms) *total_ms = 0.0;
        return LQ_OK;
    }
    if (launches) *launches = s->prof->launches[kernel_class];
    if (total_ms) *total_ms = s->prof->ms[kernel_class];
    if (reset) {
        for (int i = 0; i < lq::kProfClasses; ++i) {
            s->prof->launches[i] = 0;
            s->prof->ms[i] = 0.0;
        }
    }
    return LQ_OK;
}

} // extern "C"
