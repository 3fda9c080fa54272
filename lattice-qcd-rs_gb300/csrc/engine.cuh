// engine.cuh -- launch wrappers of the device kernels for one (D, T, COMP) instantiation.
#pragma once
#include <math.h>

#include <type_traits>

#include "adjoint.cuh"
#include "kernels.cuh"
#include "state.hpp"
#include "sweeps.cuh"

#ifndef LQ_SWEEP_SHARE1
#define LQ_SWEEP_SHARE1 1
#endif

namespace lq {

template <int D, typename T, bool COMP> struct Engine {
    static Geo<D> geo(const State &s) { return make_geo<D>(s.V, (uint32_t)s.L); }
    static dim3 link_grid(const State &s, int threads) { return dim3((s.V + threads - 1) / threads, D, 1); }
    // one thread per link, directions fastest
    static uint32_t link_blocks(const State &s, int threads) { return (uint32_t)(((uint64_t)s.V * D + threads - 1) / threads); }
    // distance in elements from the hi array to the lo array of compensated links / E-field
    static size_t ulo(const State &s) { return (size_t)tiles_of(s.V) * D * 9 * kTile; }
    static size_t elo(const State &s) { return (size_t)tiles_of(s.V) * D * 8 * kTile; }

    static cudaError_t links_from_aos(State &s, const double *d_aos, void *dst) {
        k_links_from_aos<D, T, COMP><<<link_grid(s, 128), 128, 0, s.stream>>>(d_aos, (V2<T> *)dst, s.V, ulo(s));
        return cudaGetLastError();
    }
    static cudaError_t links_to_aos(State &s, const void *src, double *d_aos) {
        k_links_to_aos<D, T, COMP><<<link_grid(s, 128), 128, 0, s.stream>>>((const V2<T> *)src, d_aos, s.V, ulo(s));
        return cudaGetLastError();
    }
    static cudaError_t links_cold(State &s, void *dst) {
        k_links_identity<D, T><<<link_grid(s, 128), 128, 0, s.stream>>>((V2<T> *)dst, s.V);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess && COMP)
            e = cudaMemsetAsync((char *)dst + s.link_bytes() / 2, 0, s.link_bytes() / 2, s.stream);
        return e;
    }
    static cudaError_t links_random(State &s, void *dst, uint64_t seed) {
        const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
        k_links_random<D, T, COMP><<<link_grid(s, 128), 128, 0, s.stream>>>((V2<T> *)dst, s.V, key, ulo(s));
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        k_normalize<D, T, COMP><<<link_grid(s, 128), 128, 0, s.stream>>>((V2<T> *)dst, geo(s), ulo(s));
        return cudaGetLastError();
    }
    static cudaError_t efield_from_aos(State &s, const double *d_aos) {
        k_efield_from_aos<D, T, COMP><<<link_blocks(s, 128), 128, 0, s.stream>>>(d_aos, (T *)s.E, s.V, elo(s));
        return cudaGetLastError();
    }
    static cudaError_t efield_hi_from_aos(State &s, const double *d_aos) {
        k_efield_from_aos<D, T, COMP, false>
            <<<link_blocks(s, 128), 128, 0, s.stream>>>(d_aos, (T *)s.E, s.V, elo(s));
        return cudaGetLastError();
    }
    static cudaError_t efield_to_aos(State &s, const void *E, double *d_aos) {
        k_efield_to_aos<D, T, COMP><<<link_blocks(s, 128), 128, 0, s.stream>>>((const T *)E, d_aos, s.V, elo(s));
        return cudaGetLastError();
    }
    // launch shape of the per-link kernels (k_md, k_md_update): 128 sites of one direction per block,
    // directions fastest (a shape of 32 sites x D directions per block measured 13% slower at 32^4)
    static dim3 md_grid_k(const State &s) { return dim3(((s.V + 127) / 128) * D, 1, 1); }
    static unsigned md_block_k() { return 128; }
    // The FP64 state: k_md_plaq + k_md_update.  Otherwise one thread per site (k_md_site) or per link
    // (k_md), as MdSite<T> selects; a drift alone has no force to share and runs per link.
    template <int M>
    static void launch_md(State &s, const void *Uin, void *Uout, const void *Ein, void *Eout, T k1, T k2, T drift) {
        if constexpr (LQ_MD_SPLIT_FP64 && std::is_same<T, double>::value && (M & MD_KICK)) {
            k_md_plaq<D, T><<<(s.V + 127) / 128, 128, 0, s.stream>>>((const V2<T> *)Uin, (T *)s.R, geo(s));
            k_md_update<D, T, COMP, M><<<md_grid_k(s), md_block_k(), 0, s.stream>>>(
                (const V2<T> *)Uin, (V2<T> *)Uout, (const T *)Ein, (T *)Eout, (const T *)s.R, geo(s), k1, k2, drift);
        } else if constexpr (MdSite<T>::on && (M & MD_KICK)) {
            k_md_site<D, T, COMP, M><<<(s.V + kMdSiteBlock - 1) / kMdSiteBlock, kMdSiteBlock, 0, s.stream>>>(
                (const V2<T> *)Uin, (V2<T> *)Uout, (const T *)Ein, (T *)Eout, geo(s), k1, k2, drift, s.block_order);
        } else {
            k_md<D, T, COMP, M><<<md_grid_k(s), md_block_k(), 0, s.stream>>>(
                (const V2<T> *)Uin, (V2<T> *)Uout, (const T *)Ein, (T *)Eout, geo(s), k1, k2, drift);
        }
    }
    // out <- scale * Im Tr(T^a U_mu(x) Sigma_mu(x)) on every link (out zeroed by the caller)
    static cudaError_t force(State &s, const void *U, void *out, double scale) {
        // kick only: the output links are never written (null)
        launch_md<MD_KICK>(s, U, nullptr, out, out, T(0), (T)scale, T(0));
        return cudaGetLastError();
    }
    static cudaError_t link_rotate(State &s, void *U, uint32_t site, int mu, int a, double angle) {
        k_link_rotate<D, T, COMP><<<1, 32, 0, s.stream>>>((V2<T> *)U, s.V, site, mu, a, (T)angle);
        return cudaGetLastError();
    }
    static cudaError_t efield_normal(State &s, uint64_t seed, uint64_t counter, double sd) {
        const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
        k_efield_normal<D, T, COMP><<<link_grid(s, 128), 128, 0, s.stream>>>(
            (T *)s.E, s.V, key, (uint32_t)counter, (uint32_t)(counter >> 32), (T)sd);
        return cudaGetLastError();
    }
    static cudaError_t md(State &s, const void *Uin, void *Uout, const void *Ein, void *Eout, int mode, double h1,
                          double h2, double dt) {
        // kick coefficient h * c_e / size with c_e = -sqrt(2 / C_A), C_A = 3
        const double ce = -sqrt(2.0 / 3.0) / s.size;
        // drift coefficient dt * sqrt(2 C_A) / size
        const double cu = sqrt(2.0 * 3.0) / s.size * dt;
        const T k1 = (T)(h1 * ce), k2 = (T)(h2 * ce), drift = (T)cu;
#define LQ_MD_CASE(M)                                                                                                  \
    case (M): launch_md<(M)>(s, Uin, Uout, Ein, Eout, k1, k2, drift); break;
        switch (mode) {
            LQ_MD_CASE(MD_KICK)
            LQ_MD_CASE(MD_DRIFT)
            LQ_MD_CASE(MD_KICK | MD_DRIFT)
            LQ_MD_CASE(MD_KICK | MD_DRIFT | MD_DRIFT_OLD_E)
            LQ_MD_CASE(MD_DRIFT | MD_EXP)
            LQ_MD_CASE(MD_KICK | MD_DRIFT | MD_EXP)
            LQ_MD_CASE(MD_KICK | MD_DRIFT | MD_DRIFT_OLD_E | MD_EXP)
            LQ_MD_CASE(MD_DRIFT | MD_EXP | MD_REUNIT)
            LQ_MD_CASE(MD_KICK | MD_DRIFT | MD_EXP | MD_REUNIT)
            LQ_MD_CASE(MD_KICK | MD_DRIFT | MD_DRIFT_OLD_E | MD_EXP | MD_REUNIT)
        default: return cudaErrorInvalidValue;
        }
#undef LQ_MD_CASE
        return cudaGetLastError();
    }
    static cudaError_t gauss(State &s, const void *U, uint32_t *n_partials) {
        const uint32_t blocks = (s.V + 255) / 256;
        k_gauss<D, T><<<blocks, 256, 0, s.stream>>>((const V2<T> *)U, (const T *)s.E, (T *)s.G, geo(s), s.partial);
        *n_partials = blocks;
        return cudaGetLastError();
    }
    // The projection runs on the hi parts only, also for compensated storage: the projected
    // field is the start momentum of a trajectory, whose low-order bits do not enter Delta H
    // (both Hamiltonians see the same start); the caller clears the lo parts afterwards.
    static cudaError_t gauss_sweep(State &s, const void *U, uint32_t *n_partials) {
        const uint32_t blocks = (s.V + 127) / 128;
        // rows whole inside the warps (L divides 32, every lane a site): the variant that takes the
        // direction-0 neighbour's step by shuffle
        const bool share0 = (kTile % s.L == 0) && (s.V % kTile == 0);
        const bool share1 = LQ_SWEEP_SHARE1 && s.L == kTile && s.V % 128 == 0 && !s.block_order.on;
        // L2 prefetch of each site's momenta and links once the hi links outgrow L2 (measured: 32^4
        // 0.132 -> 0.126 ms, 48^4 0.690 -> 0.652, 128^3 0.209 -> 0.199; 24^4, whose 96 MB of hi links
        // L2 holds, 0.0516 -> 0.0526 without the condition)
        const int pf = (uint64_t)s.V * D * 9 * sizeof(V2<T>) > kSweepPrefetchLinkBytes;
        if (share1)
            k_gauss_sweep<D, T, false, true, true><<<blocks, 128, 0, s.stream>>>(
                (const V2<T> *)U, (const T *)s.E, (T *)s.E_alt, (const T *)s.G, (T *)s.G_alt, geo(s), s.partial,
                s.block_order, pf);
        else if (share0)
            k_gauss_sweep<D, T, false, true><<<blocks, 128, 0, s.stream>>>(
                (const V2<T> *)U, (const T *)s.E, (T *)s.E_alt, (const T *)s.G, (T *)s.G_alt, geo(s), s.partial,
                s.block_order, pf);
        else
            k_gauss_sweep<D, T, false><<<blocks, 128, 0, s.stream>>>((const V2<T> *)U, (const T *)s.E, (T *)s.E_alt,
                                                                      (const T *)s.G, (T *)s.G_alt, geo(s), s.partial,
                                                                      s.block_order, pf);
        *n_partials = blocks;
        return cudaGetLastError();
    }
    static constexpr bool kAdjointProjection = std::is_same<T, double>::value;
    static cudaError_t adjoint_links(State &s, const void *U) {
        if constexpr (kAdjointProjection) {
            k_adjoint_links<D, T><<<((s.V + 127) / 128) * D, 128, 0, s.stream>>>((const V2<T> *)U, (T *)s.R, geo(s));
            return cudaGetLastError();
        } else {
            return cudaErrorNotSupported;
        }
    }
    static cudaError_t gauss_adj(State &s, uint32_t *n_partials) {
        if constexpr (kAdjointProjection) {
            const uint32_t blocks = (s.V + 255) / 256;
            k_gauss_adj<D, T><<<blocks, 256, 0, s.stream>>>((const T *)s.R, (const T *)s.E, (T *)s.G, geo(s),
                                                            s.partial);
            *n_partials = blocks;
            return cudaGetLastError();
        } else {
            return cudaErrorNotSupported;
        }
    }
    static cudaError_t gauss_step_adj(State &s) {
        if constexpr (kAdjointProjection) {
            k_gauss_step_adj<D, T><<<((s.V + 127) / 128) * D, 128, 0, s.stream>>>((const T *)s.R, (T *)s.E,
                                                                                    (const T *)s.G, geo(s));
            return cudaGetLastError();
        } else {
            return cudaErrorNotSupported;
        }
    }
    static cudaError_t gauss_to_aos(State &s, double *d_out) {
        k_gauss_to_aos<T><<<(s.V + 255) / 256, 256, 0, s.stream>>>((const T *)s.G, d_out, s.V);
        return cudaGetLastError();
    }
    static cudaError_t plaquette(State &s, const void *U, uint32_t *n_partials) {
        const uint32_t blocks = (s.V + 127) / 128;
        k_plaquette<D, T><<<blocks, 128, 0, s.stream>>>((const V2<T> *)U, geo(s), s.partial);
        *n_partials = blocks;
        return cudaGetLastError();
    }
    static cudaError_t plaquette_delta(State &s, const void *Uold, const void *Unew, uint32_t *n_partials) {
        const uint32_t blocks = (s.V + 127) / 128;
        k_plaquette_delta<D, T, COMP>
            <<<blocks, 128, 0, s.stream>>>((const V2<T> *)Uold, (const V2<T> *)Unew, geo(s), s.partial);
        *n_partials = blocks;
        return cudaGetLastError();
    }
    static cudaError_t efield_sumsq(State &s, const void *E, uint32_t *n_partials) {
        const uint32_t blocks = 1024;
        k_sum_squares<T, COMP><<<blocks, 256, 0, s.stream>>>((const T *)E, s.efield_elems(), s.partial);
        *n_partials = blocks;
        return cudaGetLastError();
    }
    static cudaError_t efield_sumsq_delta(State &s, const void *Eold, const void *Enew, uint32_t *n_partials) {
        const uint32_t blocks = 1024;
        k_sum_squares_delta<T, COMP>
            <<<blocks, 256, 0, s.stream>>>((const T *)Eold, (const T *)Enew, s.efield_elems(), s.partial);
        *n_partials = blocks;
        return cudaGetLastError();
    }
    static cudaError_t normalize(State &s, void *U) {
        k_normalize<D, T, COMP><<<link_grid(s, 128), 128, 0, s.stream>>>((V2<T> *)U, geo(s), ulo(s));
        return cudaGetLastError();
    }
    static cudaError_t finalize(State &s, int nv, uint32_t n, int offset) {
        switch (nv) {
        case 1: k_finalize<1><<<1, 1024, 0, s.stream>>>(s.partial, n, s.d_out + offset); break;
        case 2: k_finalize<2><<<1, 1024, 0, s.stream>>>(s.partial, n, s.d_out + offset); break;
        case 3: k_finalize<3><<<1, 1024, 0, s.stream>>>(s.partial, n, s.d_out + offset); break;
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }

    // ---- reverse-mode adjoint of the leap-frog (hi parts of compensated arrays)
    static dim3 md_grid(const State &s) { return dim3(((s.V + 127) / 128) * D, 1, 1); }
    static cudaError_t adj_init(State &s, const void *U, void *lamU, double scale) {
        k_adj_init<D, T><<<md_grid(s), 128, 0, s.stream>>>((const V2<T> *)U, (V2<T> *)lamU, geo(s), (T)scale);
        return cudaGetLastError();
    }
    static cudaError_t adj_kick(State &s, const void *U, const void *lamE, void *lamU, double coef) {
        k_adj_kick<D, T><<<md_grid(s), 128, 0, s.stream>>>((const V2<T> *)U, (const T *)lamE, (V2<T> *)lamU, geo(s),
                                                           (T)coef);
        return cudaGetLastError();
    }
    static cudaError_t adj_drift(State &s, const void *U, const void *E, void *lamU, void *lamE, double kappa) {
        k_adj_drift<D, T><<<md_grid(s), 128, 0, s.stream>>>((const V2<T> *)U, (const T *)E, (V2<T> *)lamU,
                                                            (T *)lamE, s.V, (T)kappa);
        return cudaGetLastError();
    }
    static cudaError_t dot(State &s, const void *a, const void *b, uint32_t *n_partials) {
        const uint32_t blocks = 1024;
        k_dot<T><<<blocks, 256, 0, s.stream>>>((const T *)a, (const T *)b, s.efield_elems(), s.partial);
        *n_partials = blocks;
        return cudaGetLastError();
    }
    // cotangent arrays (no compensated part) to the serde layouts
    static cudaError_t cot_links_to_aos(State &s, const void *lamU, double *d_aos) {
        k_links_to_aos<D, T, false><<<link_grid(s, 128), 128, 0, s.stream>>>((const V2<T> *)lamU, d_aos, s.V, 0);
        return cudaGetLastError();
    }
    static cudaError_t cot_efield_to_aos(State &s, const void *lamE, double *d_aos) {
        k_efield_to_aos<D, T, false><<<link_blocks(s, 128), 128, 0, s.stream>>>((const T *)lamE, d_aos, s.V, 0);
        return cudaGetLastError();
    }

    static cudaError_t clover_fields(State &s, const void *U, double *f_out, double *b_out) {
        k_clover_fields<D, T><<<(s.V + 127) / 128, 128, 0, s.stream>>>((const V2<T> *)U, geo(s), f_out, b_out,
                                                                         1.0 / (8.0 * s.size * s.size));
        return cudaGetLastError();
    }

    // one checkerboard class of a Metropolis (alg 0) or heat-bath (alg 1) sweep on U in place;
    // Metropolis partials (2 rows) in s.partial, their count in *n_partials
    static cudaError_t mc_sweep(State &s, void *U, int alg, int mu, int parity, double beta, uint64_t seed,
                                uint64_t sweep, int n_update, double spread, uint32_t *n_partials) {
        // k_mc_sweep maps thread t to row 2t / L and there to the sites of the class's parity along
        // x0: valid for even L only (every caller checks this too; an odd L never reaches a launch)
        if (s.L % 2 != 0) return cudaErrorInvalidValue;
        const uint32_t blocks = (s.V / 2 + 127) / 128; // one thread per site of the class
        const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
#define LQ_MC_CASE(A)                                                                                                  \
    case (A):                                                                                                          \
        k_mc_sweep<D, T, COMP, (A)><<<blocks, 128, 0, s.stream>>>((V2<T> *)U, geo(s), mu, parity, beta, key,           \
                                                                  (uint32_t)sweep, (uint32_t)(sweep >> 32), n_update, \
                                                                  spread, s.partial);                                  \
        break;
        switch (alg) {
            LQ_MC_CASE(MC_METROPOLIS)
            LQ_MC_CASE(MC_HEAT_BATH)
            LQ_MC_CASE(MC_OVERRELAX_ROTATION)
            LQ_MC_CASE(MC_OVERRELAX_REVERSE)
        default: return cudaErrorInvalidValue;
        }
#undef LQ_MC_CASE
        *n_partials = blocks;
        return cudaGetLastError();
    }

    static const Ops *table() {
        static const Ops ops = {links_from_aos, links_to_aos,  links_cold,      links_random, efield_from_aos,
                                efield_to_aos,  efield_normal, md,              gauss,        gauss_sweep,
                                gauss_to_aos,
                                kAdjointProjection ? adjoint_links : nullptr,
                                kAdjointProjection ? gauss_adj : nullptr,
                                kAdjointProjection ? gauss_step_adj : nullptr,
                                plaquette,     plaquette_delta, efield_sumsq, efield_sumsq_delta,
                                normalize,      finalize,       force,         link_rotate,
                                adj_init,       adj_kick,       adj_drift,     dot,
                                cot_links_to_aos, cot_efield_to_aos, clover_fields, mc_sweep, efield_hi_from_aos};
        return &ops;
    }
};

} // namespace lq
