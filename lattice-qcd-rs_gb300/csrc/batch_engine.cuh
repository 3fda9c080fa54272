// batch_engine.cuh -- batched kernels over many ensembles (one launch covers every ensemble
// through the chunk table) and their launch wrappers for one (D, T, COMP) instantiation.
//
// Each kernel is persistent in form: block b takes work items b, b + gridDim.x, ... of the
// chunk table (x D directions for per-link kernels), so the autotuner can run it with one
// block per item or with a grid of a few waves of resident blocks.  The per-site and
// per-link arithmetic is the single-lattice kernels' own (md_link, sweep_site, ...), so an
// ensemble of a batch evolves exactly as a lattice run alone does; reductions keep one
// partial per 128-site chunk, the single-lattice kernels' per-block partials.
#pragma once
#include <math.h>

#include "batch.hpp"
#include "kernels.cuh"

namespace lq {

template <typename T> struct BView {
    V2<T> *U[3];
    T *E[2];
    T *G[2];
    size_t ulo, elo; // hi -> lo distance of links / E-field, in elements
    const BatchEns *ens;
    BatchRun *run;
    const uint2 *chunks;
    const uint64_t *keys;
    double *partial; // rows of n_chunks
    uint32_t n_chunks;
};

// buffer selection by value: indexing the kernel-parameter arrays with a runtime index would
// copy the whole view to local memory
template <typename T> __device__ __forceinline__ V2<T> *sel_u(const BView<T> &v, int r) {
    return r == 0 ? v.U[0] : (r == 1 ? v.U[1] : v.U[2]);
}
template <typename T> __device__ __forceinline__ T *sel_e(const BView<T> &v, int r) { return r == 0 ? v.E[0] : v.E[1]; }
template <typename T> __device__ __forceinline__ T *sel_g(const BView<T> &v, int r) { return r == 0 ? v.G[0] : v.G[1]; }

template <int D> __device__ __forceinline__ Geo<D> geo_of(const BatchEns &e) {
    Geo<D> g;
    g.V = e.V;
    g.L = e.L;
#pragma unroll
    for (int i = 0; i < 4; ++i) g.stride[i] = e.stride[i];
    g.lm = e.lm;
    g.ls = e.ls;
    return g;
}

// work item w of a per-link kernel: order 0 directions fastest, 1 chunks fastest
template <int D>
__device__ __forceinline__ void link_item(uint32_t w, uint32_t n_chunks, int order, uint32_t &chunk, int &mu) {
    if (order == 0) {
        chunk = w / D;
        mu = (int)(w % D);
    } else {
        chunk = w % n_chunks;
        mu = (int)(w / n_chunks);
    }
}

__device__ __forceinline__ uint2 key_of(uint64_t k) { return make_uint2((uint32_t)k, (uint32_t)(k >> 32)); }

// a table coefficient in the arithmetic type
template <typename T> __device__ __forceinline__ T coef(float f, double d) {
    if constexpr (sizeof(T) == 4) return f;
    else return d;
}

// ------------------------------------------------------------------ trajectory kernels
// E[eout] <- Normal(0, 0.5 / beta) per ensemble, Philox key keys[e] and counter run[e].counter
// (k_efield_normal's stream for that seed and counter); also opens the trajectory's
// projection bookkeeping of every ensemble.
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_normal_batch(BView<T> v, int eout, int order) {
    const uint32_t n_work = v.n_chunks * D;
    for (uint32_t w = blockIdx.x; w < n_work; w += gridDim.x) {
        uint32_t chunk;
        int mu;
        link_item<D>(w, v.n_chunks, order, chunk, mu);
        const uint2 c = v.chunks[chunk];
        const BatchEns &en = v.ens[c.x];
        const uint32_t site = c.y + threadIdx.x;
        if (chunk == en.chunk0 && mu == 0 && threadIdx.x == 0) {
            BatchRun &r = v.run[c.x];
            r.converged = 0;
            r.steps = 0;
            r.status = LQ_OK;
        }
        if (site >= en.V) continue;
        const unsigned long long ctr = v.run[c.x].counter;
        const size_t eb = (size_t)en.tile0 * (D * 8 * kTile);
        efield_normal_link<D, T, COMP>(sel_e(v, eout) + eb, site, mu, key_of(v.keys[c.x]), (uint32_t)ctr,
                                       (uint32_t)(ctr >> 32), coef<T>(en.sd_f, en.sd_d), v.elo);
    }
}

// G[gout] <- gauss(E[ein], U[cur]) (the projection's start; residuals are not needed)
template <int D, typename T>
__global__ void __launch_bounds__(128) k_gauss_batch(BView<T> v, int ein, int gout) {
    for (uint32_t chunk = blockIdx.x; chunk < v.n_chunks; chunk += gridDim.x) {
        const uint2 c = v.chunks[chunk];
        const BatchEns &en = v.ens[c.x];
        const uint32_t site = c.y + threadIdx.x;
        if (site >= en.V) continue;
        const int cur = v.run[c.x].cur;
        const size_t ub = (size_t)en.tile0 * (D * 9 * kTile), eb = (size_t)en.tile0 * (D * 8 * kTile),
                     gb = (size_t)en.tile0 * (9 * kTile);
        (void)gauss_site<D, T>(sel_u(v, cur) + ub, sel_e(v, ein) + eb, sel_g(v, gout) + gb, geo_of<D>(en), site);
    }
}

// one projection sweep (E[ein], G[gin]) -> (E[eout], G[gout]) with per-chunk residuals in
// partial row 0; ensembles whose projection has finished are skipped.  Hi parts only.
template <int D, typename T>
__global__ void __launch_bounds__(128, MinBlocks<T>::sweep) k_sweep_batch(BView<T> v, int ein, int eout, int gin,
                                                                          int gout, int pf) {
    for (uint32_t chunk = blockIdx.x; chunk < v.n_chunks; chunk += gridDim.x) {
        const uint2 c = v.chunks[chunk];
        if (v.run[c.x].converged) continue; // uniform over the block
        const BatchEns &en = v.ens[c.x];
        const uint32_t site = c.y + threadIdx.x;
        double r[1] = {0.0};
        if (site < en.V) {
            const int cur = v.run[c.x].cur;
            const size_t ub = (size_t)en.tile0 * (D * 9 * kTile), eb = (size_t)en.tile0 * (D * 8 * kTile),
                         gb = (size_t)en.tile0 * (9 * kTile);
            r[0] = sweep_site<D, T, false>(sel_u(v, cur) + ub, sel_e(v, ein) + eb, sel_e(v, eout) + eb, sel_g(v, gin) + gb,
                                           sel_g(v, gout) + gb, geo_of<D>(en), site, v.elo, nullptr, pf != 0);
        }
        block_reduce_store<1>(r, v.partial, chunk, v.n_chunks);
        __syncthreads();
    }
}

// After a sweep: one block per ensemble sums its chunk residuals (k_finalize's order) and
// applies project_to_gauss's test (src/field.rs:1265-1294) -- residual <= eps V 320 ends the
// projection, NaN fails it, and the step limit stops it; the last block to finish sets the
// loop flag (and the graph's while condition) to whether any projection is still running.
static __global__ void __launch_bounds__(1024) k_check_batch(const BatchEns *__restrict__ ens, BatchRun *run,
                                                      const double *__restrict__ partial, int steps_added,
                                                      int max_steps, double eps, unsigned int *done, int *flag,
                                                      cudaGraphConditionalHandle handle, int use_handle) {
    const int e = blockIdx.x;
    const BatchEns en = ens[e];
    const int finished = run[e].converged;
    if (!finished) {
        double v[1] = {0.0};
        for (uint32_t k = threadIdx.x; k < en.nchunks; k += blockDim.x) v[0] += partial[en.chunk0 + k];
        __shared__ double res[1];
        block_reduce_store<1>(v, res, 0, 1);
        __syncthreads();
        if (threadIdx.x == 0) {
            BatchRun &r = run[e];
            r.steps += steps_added;
            const double val = res[0];
            const double threshold = eps * (double)((uint64_t)en.V * 4 * 8 * 10);
            if (isnan(val)) {
                r.status = LQ_ERR_GAUSS_PROJECTION;
                r.converged = 1;
            } else if (val <= threshold) {
                r.converged = 1;
            } else if (max_steps > 0 && r.steps + 4 > max_steps) {
                r.status = LQ_ERR_NOT_CONVERGED;
                r.converged = 1;
            }
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int ticket = atomicAdd(done, 1u);
        if (ticket == gridDim.x - 1) {
            int any = 0;
            volatile const BatchRun *vr = run;
            for (unsigned int i = 0; i < gridDim.x; ++i) any |= (vr[i].converged == 0);
            *flag = any;
            if (use_handle) cudaGraphSetConditional(handle, any ? 1u : 0u);
            *done = 0u;
            __threadfence();
        }
    }
}

template <int D, typename T, bool COMP, int MODE>
__global__ void __launch_bounds__(128, MinBlocks<T>::md) k_md_batch(BView<T> v, int rin, int rout, int ein,
                                                                    int eout, int k1_on, int order) {
    const uint32_t n_work = v.n_chunks * D;
    for (uint32_t w = blockIdx.x; w < n_work; w += gridDim.x) {
        uint32_t chunk;
        int mu;
        link_item<D>(w, v.n_chunks, order, chunk, mu);
        const uint2 c = v.chunks[chunk];
        const BatchEns &en = v.ens[c.x];
        const uint32_t site = c.y + threadIdx.x;
        if (site >= en.V) continue;
        const int cur = v.run[c.x].cur;
        const size_t ub = (size_t)en.tile0 * (D * 9 * kTile), eb = (size_t)en.tile0 * (D * 8 * kTile);
        const T kh = coef<T>(en.kh_f, en.kh_d);
        md_link<D, T, COMP, MODE>(sel_u(v, (cur + rin) % 3) + ub, sel_u(v, (cur + rout) % 3) + ub, sel_e(v, ein) + eb,
                                  sel_e(v, eout) + eb, geo_of<D>(en), site, mu, k1_on ? kh : T(0), kh,
                                  coef<T>(en.dr_f, en.dr_d), v.ulo, v.elo);
    }
}

// the same step with one thread per site (md_site), as the single-lattice kernel of this precision runs it
template <int D, typename T, bool COMP, int MODE>
__global__ void __launch_bounds__(kMdSiteBlock, MinBlocks<T>::md_site)
    k_md_site_batch(BView<T> v, int rin, int rout, int ein, int eout, int k1_on) {
    static_assert(kChunk == kMdSiteBlock, "one chunk per block");
    __shared__ T fs[(D - 1) * 8][kMdSiteBlock];
    for (uint32_t w = blockIdx.x; w < v.n_chunks; w += gridDim.x) {
        const uint2 c = v.chunks[w];
        const BatchEns &en = v.ens[c.x];
        const uint32_t site = c.y + threadIdx.x;
        if (site >= en.V) continue;
        const int cur = v.run[c.x].cur;
        const size_t ub = (size_t)en.tile0 * (D * 9 * kTile), eb = (size_t)en.tile0 * (D * 8 * kTile);
        const T kh = coef<T>(en.kh_f, en.kh_d);
        md_site<D, T, COMP, MODE>(sel_u(v, (cur + rin) % 3) + ub, sel_u(v, (cur + rout) % 3) + ub, sel_e(v, ein) + eb,
                                  sel_e(v, eout) + eb, geo_of<D>(en), site, k1_on ? kh : T(0), kh,
                                  coef<T>(en.dr_f, en.dr_d), v.ulo, v.elo, fs, threadIdx.x);
    }
}

// partial row 0 <- per-chunk sum Re Tr[P(U[r_new]) - P(U[r_old])]
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_plaquette_delta_batch(BView<T> v, int r_old, int r_new) {
    for (uint32_t chunk = blockIdx.x; chunk < v.n_chunks; chunk += gridDim.x) {
        const uint2 c = v.chunks[chunk];
        const BatchEns &en = v.ens[c.x];
        const uint32_t site = c.y + threadIdx.x;
        double r[1] = {0.0};
        if (site < en.V) {
            const int cur = v.run[c.x].cur;
            const size_t ub = (size_t)en.tile0 * (D * 9 * kTile);
            r[0] = plaquette_delta_site<D, T, COMP>(sel_u(v, (cur + r_old) % 3) + ub, sel_u(v, (cur + r_new) % 3) + ub,
                                                    geo_of<D>(en), site, v.ulo);
        }
        block_reduce_store<1>(r, v.partial, chunk, v.n_chunks);
        __syncthreads();
    }
}

// partial row 1 <- per-chunk sum (e' - e)(e' + e) of E[e_old] -> E[e_new]
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_sumsq_delta_batch(BView<T> v, int e_old, int e_new) {
    for (uint32_t chunk = blockIdx.x; chunk < v.n_chunks; chunk += gridDim.x) {
        const uint2 c = v.chunks[chunk];
        const BatchEns &en = v.ens[c.x];
        const uint32_t site = c.y + threadIdx.x;
        T acc = T(0);
        if (site < en.V) {
            const size_t eb = (size_t)en.tile0 * (D * 8 * kTile);
            const T *eo = sel_e(v, e_old) + eb;
            const T *ew = sel_e(v, e_new) + eb;
#pragma unroll
            for (int mu = 0; mu < D; ++mu) {
                const size_t i = tix(site, D * 8, mu * 8);
                T a[8], b[8], al[8], bl[8];
                load_efield<T>(eo, i, a);
                load_efield<T>(ew, i, b);
                if (COMP) {
                    load_efield<T>(eo + v.elo, i, al);
                    load_efield<T>(ew + v.elo, i, bl);
                }
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    T d = b[k] - a[k];
                    if (COMP) d += bl[k] - al[k];
                    acc = fma(d, a[k] + b[k], acc);
                }
            }
        }
        double r[1] = {(double)acc};
        block_reduce_store<1>(r, v.partial + v.n_chunks, chunk, v.n_chunks);
        __syncthreads();
    }
}

// partial rows 0..2 <- per-chunk plaquette sums of U[role] (k_plaquette's three rows)
template <int D, typename T>
__global__ void __launch_bounds__(128) k_plaquette_batch(BView<T> v, int role) {
    for (uint32_t chunk = blockIdx.x; chunk < v.n_chunks; chunk += gridDim.x) {
        const uint2 c = v.chunks[chunk];
        const BatchEns &en = v.ens[c.x];
        const uint32_t site = c.y + threadIdx.x;
        double r[3] = {0.0, 0.0, 0.0};
        if (site < en.V) {
            const int cur = v.run[c.x].cur;
            plaquette_site<D, T>(sel_u(v, (cur + role) % 3) + (size_t)en.tile0 * (D * 9 * kTile), geo_of<D>(en), site,
                                 r);
        }
        block_reduce_store<3>(r, v.partial, chunk, v.n_chunks);
        __syncthreads();
    }
}

// One block per ensemble: Delta H from the two partial rows, the Metropolis test with a
// uniform from the ensemble's Philox stream, the accepted links become the state.
//   Delta H = -beta/3 sum Re Tr[P' - P] + beta/2 sum (e'^2 - e^2)
//   p = clamp(exp(-Delta H), 0, 1) (probability_of_replacement, hybrid_monte_carlo.rs:584-589)
static __global__ void __launch_bounds__(1024) k_accept_batch(const BatchEns *__restrict__ ens, BatchRun *run,
                                                       const uint64_t *__restrict__ keys,
                                                       const double *__restrict__ partial, uint32_t n_chunks,
                                                       int r_final, BatchResult *results, int result_rows) {
    const int e = blockIdx.x;
    const BatchEns en = ens[e];
    double v[2] = {0.0, 0.0};
    for (uint32_t k = threadIdx.x; k < en.nchunks; k += blockDim.x) {
        v[0] += partial[en.chunk0 + k];
        v[1] += partial[n_chunks + en.chunk0 + k];
    }
    __shared__ double res[2];
    block_reduce_store<2>(v, res, 0, 1);
    __syncthreads();
    if (threadIdx.x != 0) return;
    BatchRun &r = run[e];
    const double hu = -res[0] / 3.0 * en.beta;
    const double he = res[1] / 2.0 * en.beta;
    const double dh = hu + he;
    double p = fmax(fmin(exp(-dh), 1.0), 0.0);
    const unsigned long long ctr = r.counter;
    const uint4 q = philox4x32_10(make_uint4(0xFFFFFFFFu, (uint32_t)ctr, (uint32_t)(ctr >> 32), 4u), key_of(keys[e]));
    const double u = u01_53(q.x, q.y);
    int acc = 0;
    if (r.status == LQ_OK) {
        acc = (p >= 1.0 || u < p) ? 1 : 0;
        if (acc) r.cur = (r.cur + r_final) % 3;
    } else {
        p = 0.0;
    }
    if (r.row >= 0 && r.row < result_rows) {
        BatchResult out;
        out.delta_h = dh;
        out.prob = p;
        out.uniform = u;
        out.plaq_re = 0.0;
        out.plaq_im = 0.0;
        out.accepted = acc;
        out.gauss_steps = r.steps;
        out.status = r.status;
        out.pad = 0;
        results[(size_t)r.row * gridDim.x + e] = out;
    }
    r.row += 1;
    r.counter += 1;
}

// one block per ensemble: plaquette rows -> sums (mode 0: d_out[3e + i]) or the average trace
// of the last recorded trajectory (mode 1: results[row - 1])
static __global__ void __launch_bounds__(1024) k_plaquette_finish_batch(const BatchEns *__restrict__ ens,
                                                                 const BatchRun *__restrict__ run,
                                                                 const double *__restrict__ partial,
                                                                 uint32_t n_chunks, int dim, double *d_out,
                                                                 BatchResult *results, int result_rows) {
    const int e = blockIdx.x;
    const BatchEns en = ens[e];
    double v[3] = {0.0, 0.0, 0.0};
    for (uint32_t k = threadIdx.x; k < en.nchunks; k += blockDim.x)
#pragma unroll
        for (int i = 0; i < 3; ++i) v[i] += partial[(size_t)i * n_chunks + en.chunk0 + k];
    __shared__ double res[3];
    block_reduce_store<3>(v, res, 0, 1);
    __syncthreads();
    if (threadIdx.x != 0) return;
    if (d_out) {
#pragma unroll
        for (int i = 0; i < 3; ++i) d_out[3 * e + i] = res[i];
    } else {
        const int row = run[e].row - 1;
        if (row >= 0 && row < result_rows) {
            const double n_plaq = (double)((uint64_t)en.V * (uint64_t)((dim * (dim - 1)) / 2));
            results[(size_t)row * gridDim.x + e].plaq_re = res[1] / n_plaq;
            results[(size_t)row * gridDim.x + e].plaq_im = res[2] / n_plaq;
        }
    }
}

// ------------------------------------------------------------------ launch wrappers
template <int D, typename T, bool COMP> struct BatchEngine {
    static BView<T> view(Batch &b) {
        BView<T> v;
        for (int i = 0; i < 3; ++i) v.U[i] = (V2<T> *)b.U[i];
        for (int i = 0; i < 2; ++i) {
            v.E[i] = (T *)b.E[i];
            v.G[i] = (T *)b.G[i];
        }
        v.ulo = b.link_elems();
        v.elo = b.efield_elems();
        v.ens = b.ens;
        v.run = b.run;
        v.chunks = b.chunks;
        v.keys = b.keys;
        v.partial = b.partial;
        v.n_chunks = b.n_chunks;
        return v;
    }
    static uint32_t grid(const Batch &b, int cls, uint32_t n_work) {
        const uint32_t g = b.shape[cls].grid;
        return (g == 0 || g > n_work) ? n_work : g;
    }
    // per-ensemble element offsets
    static size_t ub(const Batch &b, int e) { return (size_t)b.ens_h[e].tile0 * (D * 9 * kTile); }
    static dim3 link_grid(const Batch &b, int e) { return dim3((b.ens_h[e].V + 127) / 128, D, 1); }
    static Geo<D> geo_h(const Batch &b, int e) { return make_geo<D>(b.ens_h[e].V, b.ens_h[e].L); }
    // per-ensemble operations on link buffer `buf` (the ensemble's state buffer, run[e].cur)
    static cudaError_t links_from_aos(Batch &b, int e, int buf, const double *d_aos) {
        k_links_from_aos<D, T, COMP><<<link_grid(b, e), 128, 0, b.stream>>>(d_aos, (V2<T> *)b.U[buf] + ub(b, e),
                                                                              b.ens_h[e].V, b.link_elems());
        return cudaGetLastError();
    }
    static cudaError_t links_to_aos(Batch &b, int e, int buf, double *d_aos) {
        k_links_to_aos<D, T, COMP><<<link_grid(b, e), 128, 0, b.stream>>>((const V2<T> *)b.U[buf] + ub(b, e), d_aos,
                                                                            b.ens_h[e].V, b.link_elems());
        return cudaGetLastError();
    }
    static cudaError_t links_random(Batch &b, int e, int buf, uint64_t seed) {
        const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
        V2<T> *U = (V2<T> *)b.U[buf] + ub(b, e);
        k_links_random<D, T, COMP><<<link_grid(b, e), 128, 0, b.stream>>>(U, b.ens_h[e].V, key, b.link_elems());
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        k_normalize<D, T, COMP><<<link_grid(b, e), 128, 0, b.stream>>>(U, geo_h(b, e), b.link_elems());
        return cudaGetLastError();
    }
    static cudaError_t links_cold(Batch &b, int e, int buf) {
        V2<T> *U = (V2<T> *)b.U[buf] + ub(b, e);
        k_links_identity<D, T><<<link_grid(b, e), 128, 0, b.stream>>>(U, b.ens_h[e].V);
        cudaError_t err = cudaGetLastError();
        if (err == cudaSuccess && COMP)
            err = cudaMemsetAsync(U + b.link_elems(), 0,
                                  (size_t)tiles_of(b.ens_h[e].V) * D * 9 * kTile * sizeof(V2<T>), b.stream);
        return err;
    }
    static cudaError_t normalize(Batch &b, int e, int buf) {
        k_normalize<D, T, COMP>
            <<<link_grid(b, e), 128, 0, b.stream>>>((V2<T> *)b.U[buf] + ub(b, e), geo_h(b, e), b.link_elems());
        return cudaGetLastError();
    }

    static cudaError_t normal(Batch &b, int eout) {
        const uint32_t n = b.n_chunks * D;
        k_normal_batch<D, T, COMP><<<grid(b, BK_NORMAL, n), kChunk, 0, b.stream>>>(view(b), eout, b.shape[BK_NORMAL].order);
        return cudaGetLastError();
    }
    static cudaError_t gauss(Batch &b, int ein, int gout) {
        k_gauss_batch<D, T><<<grid(b, BK_GAUSS, b.n_chunks), kChunk, 0, b.stream>>>(view(b), ein, gout);
        return cudaGetLastError();
    }
    static cudaError_t sweep(Batch &b, int ein, int eout, int gin, int gout) {
        // the single lattice's rule over the hi links of all ensembles
        const int pf = b.total_links * 9 * sizeof(V2<T>) > kSweepPrefetchLinkBytes;
        k_sweep_batch<D, T><<<grid(b, BK_SWEEP, b.n_chunks), kChunk, 0, b.stream>>>(view(b), ein, eout, gin, gout, pf);
        return cudaGetLastError();
    }
    static cudaError_t check(Batch &b, int steps_added, int max_steps, cudaGraphConditionalHandle h, int use_handle) {
        const double eps = sizeof(T) == 8 ? 2.220446049250313e-16 : 1.1920928955078125e-07;
        k_check_batch<<<b.n_ens, 1024, 0, b.stream>>>(b.ens, b.run, b.partial, steps_added, max_steps, eps, b.done,
                                                      b.flag, h, use_handle);
        return cudaGetLastError();
    }
    template <int M> static void launch_md(Batch &b, int rin, int rout, int ein, int eout, int k1_on) {
        const BView<T> v = view(b);
        if constexpr (MdSite<T>::on && (M & MD_KICK)) {
            k_md_site_batch<D, T, COMP, M>
                <<<grid(b, BK_MD, b.n_chunks), kChunk, 0, b.stream>>>(v, rin, rout, ein, eout, k1_on);
        } else {
            k_md_batch<D, T, COMP, M><<<grid(b, BK_MD, b.n_chunks * D), kChunk, 0, b.stream>>>(
                v, rin, rout, ein, eout, k1_on, b.shape[BK_MD].order);
        }
    }
    static cudaError_t md(Batch &b, int rin, int rout, int ein, int eout, int mode, int k1_on) {
#define LQ_MDB_CASE(M)                                                                                                 \
    case (M): launch_md<(M)>(b, rin, rout, ein, eout, k1_on); break;
        switch (mode) {
            LQ_MDB_CASE(MD_KICK)
            LQ_MDB_CASE(MD_KICK | MD_DRIFT)
            LQ_MDB_CASE(MD_KICK | MD_DRIFT | MD_EXP)
            LQ_MDB_CASE(MD_KICK | MD_DRIFT | MD_EXP | MD_REUNIT)
        default: return cudaErrorInvalidValue;
        }
#undef LQ_MDB_CASE
        return cudaGetLastError();
    }
    static cudaError_t plaquette_delta(Batch &b, int r_old, int r_new) {
        k_plaquette_delta_batch<D, T, COMP>
            <<<grid(b, BK_PLAQ_DELTA, b.n_chunks), kChunk, 0, b.stream>>>(view(b), r_old, r_new);
        return cudaGetLastError();
    }
    static cudaError_t sumsq_delta(Batch &b, int e_old, int e_new) {
        k_sumsq_delta_batch<D, T, COMP>
            <<<grid(b, BK_SUMSQ_DELTA, b.n_chunks), kChunk, 0, b.stream>>>(view(b), e_old, e_new);
        return cudaGetLastError();
    }
    static cudaError_t accept(Batch &b, int r_final) {
        k_accept_batch<<<b.n_ens, 1024, 0, b.stream>>>(b.ens, b.run, b.keys, b.partial, b.n_chunks, r_final, b.results,
                                                       b.result_rows);
        return cudaGetLastError();
    }
    static cudaError_t plaquette(Batch &b, int role) {
        k_plaquette_batch<D, T><<<grid(b, BK_PLAQUETTE, b.n_chunks), kChunk, 0, b.stream>>>(view(b), role);
        return cudaGetLastError();
    }
    static cudaError_t plaquette_sums(Batch &b, double *d_out) {
        cudaError_t err = plaquette(b, 0);
        if (err != cudaSuccess) return err;
        k_plaquette_finish_batch<<<b.n_ens, 1024, 0, b.stream>>>(b.ens, b.run, b.partial, b.n_chunks, D, d_out,
                                                                 nullptr, 0);
        return cudaGetLastError();
    }
    static cudaError_t record_plaquette(Batch &b) {
        cudaError_t err = plaquette(b, 0);
        if (err != cudaSuccess) return err;
        k_plaquette_finish_batch<<<b.n_ens, 1024, 0, b.stream>>>(b.ens, b.run, b.partial, b.n_chunks, D, nullptr,
                                                                 b.results, b.result_rows);
        return cudaGetLastError();
    }
    static int occupancy(int cls) {
        int n = 0;
        cudaError_t err = cudaSuccess;
        switch (cls) {
        case BK_MD:
            if constexpr (MdSite<T>::on)
                err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_md_site_batch<D, T, COMP, MD_KICK | MD_DRIFT>,
                                                                    kChunk, 0);
            else
                err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_md_batch<D, T, COMP, MD_KICK | MD_DRIFT>,
                                                                    kChunk, 0);
            break;
        case BK_SWEEP: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_batch<D, T>, kChunk, 0); break;
        case BK_GAUSS: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_gauss_batch<D, T>, kChunk, 0); break;
        case BK_PLAQ_DELTA:
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_plaquette_delta_batch<D, T, COMP>, kChunk, 0);
            break;
        case BK_SUMSQ_DELTA:
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sumsq_delta_batch<D, T, COMP>, kChunk, 0);
            break;
        case BK_NORMAL:
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_normal_batch<D, T, COMP>, kChunk, 0);
            break;
        case BK_PLAQUETTE:
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_plaquette_batch<D, T>, kChunk, 0);
            break;
        default: return 0;
        }
        if (err != cudaSuccess) {
            (void)cudaGetLastError();
            return 0;
        }
        return n;
    }

    static const BatchOps *table() {
        static const BatchOps ops = {links_from_aos, links_to_aos, links_random,    links_cold,   normalize,
                                     normal,         gauss,        sweep,           check,        md,
                                     plaquette_delta, sumsq_delta, accept,          plaquette,    plaquette_sums,
                                     record_plaquette, occupancy};
        return &ops;
    }
};

} // namespace lq
