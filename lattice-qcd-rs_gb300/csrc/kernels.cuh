// kernels.cuh -- device kernels of the HMC molecular-dynamics path, templated on the
// lattice dimension D (2, 3, 4), the arithmetic type T (double or float) and COMP, which
// selects compensated storage: every stored real is a pair (hi, lo) of T, hi + lo, updated
// with error-free two-sums, while all products use hi only.
//
// Device layout (tiled structure of arrays, see tix() in su3.cuh: 32-site tiles, all planes
// of a tile contiguous, plane p of site s at ((s/32)*P + p)*32 + s%32):
//   links  U : vec2<T>, P = D*9 planes, plane mu*9 + k holds entry k = row*3 + col of U_mu;
//              with COMP the lo parts follow as a second array of the same shape
//   efield E : T, P = D*8 planes, planes mu*8 .. mu*8+7 hold e^a of E_mu, packed per site into
//              16-byte vectors (efield_off / load_efield) (+ lo array with COMP)
//   gauss  G : T, P = 9 planes, Hermitian G(x): real diagonal + upper off-diagonal; in the FP64
//              projection 10 planes, the 9 components of G and a pad, packed like E
//   scratch  : FP64 only, D*82 planes per site: the projection's per-link transport tables, and
//              between projections the MD step's per-link force parts
// Sites are linearised x_0 fastest as in the reference (src/lattice.rs:909-916), so the
// +-mu neighbour of a site is +-L^mu with periodic wrap.  Arrays are padded to whole tiles;
// padded sites are never written by the kernels and stay zero.
#pragma once
#include "block_order.hpp"
#include "su3.cuh"

namespace lq {

template <int D> struct Geo {
    uint32_t V;         // number of sites L^D
    uint32_t L;         // points per direction
    uint32_t stride[4]; // L^mu
    uint32_t lm, ls;    // division by L: n / L = (mulhi(n, lm) + n) >> ls (divisor_magic)
};

// Multiplier m and shift s of the division by d >= 1 for every 32-bit dividend n, by the round-up
// method of Granlund and Montgomery ("Division by invariant integers using multiplication", 1994):
// s = ceil(log2 d), m = floor(2^32 (2^s - d) / d) + 1, n / d = (mulhi(n, m) + n) >> s with the
// sum taken in 64 bits.  A few integer instructions instead of the general division.
__host__ __device__ inline void divisor_magic(uint32_t d, uint32_t &m, uint32_t &s) {
    s = 0;
    while ((1ull << s) < d) ++s;
    m = (uint32_t)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
}

template <int D> __host__ __device__ inline Geo<D> make_geo(uint32_t V, uint32_t L) {
    Geo<D> g;
    g.V = V;
    g.L = L;
    uint32_t st = 1;
    for (int i = 0; i < 4; ++i) {
        g.stride[i] = st;
        if (i < D) st *= L;
    }
    divisor_magic(L, g.lm, g.ls);
    return g;
}

template <int D> __device__ __forceinline__ uint32_t div_by_L(const Geo<D> &g, uint32_t n) {
    return (uint32_t)(((uint64_t)__umulhi(n, g.lm) + n) >> g.ls);
}

// coordinates of a site, c[i] = (site / L^i) % L, one division by L per direction
template <int D> __device__ __forceinline__ void site_coords(const Geo<D> &g, uint32_t site, uint32_t *c) {
    uint32_t r = checked_site(site, g.V);
#pragma unroll
    for (int i = 0; i < D; ++i) {
        const uint32_t q = div_by_L(g, r);
        c[i] = r - q * g.L;
        r = q;
    }
}
// neighbour of `site` (whose coordinate along mu is cmu) in +mu / -mu, periodic
template <int D>
__device__ __forceinline__ uint32_t fwd(const Geo<D> &g, uint32_t site, uint32_t cmu, int mu) {
    return checked_site((cmu == g.L - 1) ? site - (g.L - 1) * g.stride[mu] : site + g.stride[mu], g.V);
}
template <int D>
__device__ __forceinline__ uint32_t bwd(const Geo<D> &g, uint32_t site, uint32_t cmu, int mu) {
    return checked_site((cmu == 0) ? site + (g.L - 1) * g.stride[mu] : site - g.stride[mu], g.V);
}

template <typename T> using V2 = typename vec2_t<T>::type;

// Minimum resident blocks per SM requested from the register allocator for the FP32 forms
// of the MD kernel and the projection sweep (1: no request).  Measured on GB300 at 32^4: the MD
// kernel is best at 5 (96 registers; 4: +5 %, 6: +1 %), the sweep at 4 (128 registers, no spills;
// 5: +1 %, 6: +3 %).  The FP64 forms keep the allocator's choice: their working set needs about
// twice the registers.
#ifndef LQ_MD_MIN_BLOCKS
#define LQ_MD_MIN_BLOCKS 5
#endif
#ifndef LQ_SWEEP_MIN_BLOCKS
#define LQ_SWEEP_MIN_BLOCKS 4
#endif

// The MD step runs one thread per site (k_md_site, the plaquettes shared between a site's links) or
// one thread per link (k_md); LQ_MD_SITE_FP64 / LQ_MD_SITE_FP32 choose per precision.  The FP64
// state runs it as two launches (k_md_plaq + k_md_update, every plaquette formed once) unless
// LQ_MD_SPLIT_FP64 is 0.
#ifndef LQ_MD_SPLIT_FP64
#define LQ_MD_SPLIT_FP64 1
#endif
#ifndef LQ_MD_SITE_FP64
#define LQ_MD_SITE_FP64 1
#endif
#ifndef LQ_MD_SITE_FP32
#define LQ_MD_SITE_FP32 1
#endif
#ifndef LQ_MD_SITE_MIN_BLOCKS
#define LQ_MD_SITE_MIN_BLOCKS 4
#endif
#ifndef LQ_MD_SITE_MIN_BLOCKS_FP64
#define LQ_MD_SITE_MIN_BLOCKS_FP64 1
#endif
constexpr int kMdSiteBlock = 128;
// L2 prefetch of the site kernel's read-once update data at the start of each direction (measured at
// 32^4: mixed 0.375 -> 0.365 ms, f32 0.310 -> 0.301 ms per kick+drift launch, bitwise the same fields)
#ifndef LQ_MD_PREFETCH
#define LQ_MD_PREFETCH 1
#endif
// The projection sweep prefetches each site's momenta and links to L2 when the hi links of the lattice
// (of all ensembles, in a batch) exceed this many bytes: the GB300 L2 is 129 MB.
#ifndef LQ_SWEEP_PREFETCH_LINK_BYTES
#define LQ_SWEEP_PREFETCH_LINK_BYTES (128ull << 20)
#endif
constexpr uint64_t kSweepPrefetchLinkBytes = LQ_SWEEP_PREFETCH_LINK_BYTES;
template <typename T> struct MdSite {
    static constexpr bool on = sizeof(T) == 8 ? LQ_MD_SITE_FP64 : LQ_MD_SITE_FP32;
};
template <typename T> struct MinBlocks {
    static constexpr int md_site = sizeof(T) == 4 ? LQ_MD_SITE_MIN_BLOCKS : LQ_MD_SITE_MIN_BLOCKS_FP64;
    static constexpr int md = sizeof(T) == 4 ? LQ_MD_MIN_BLOCKS : 1;
    static constexpr int sweep = sizeof(T) == 4 ? LQ_SWEEP_MIN_BLOCKS : 1;
};
// The single-lattice plaquette difference in FP32 at D = 4 fits three blocks per SM without
// spilling (168 registers; two at the allocator's own choice of 172); D = 2, 3 and the batched
// kernel spill under the same cap and keep the allocator's choice.
#ifndef LQ_DELTA_MIN_BLOCKS
#define LQ_DELTA_MIN_BLOCKS 3
#endif
template <int D, typename T> struct MinBlocksDelta {
    static constexpr int value = (sizeof(T) == 4 && D == 4) ? LQ_DELTA_MIN_BLOCKS : 1;
};

// a + b and a - b rounded to nearest, never fused with a product that computed an operand
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// (hi, lo) += d: two-sum of hi and d, error folded into lo, pair renormalised (Knuth's TwoSum
// followed by Dekker's FastTwoSum).  Every add is an explicit rounded add: d is usually a product
// (k f, drift x), and an add contracted with it into an FMA would break the two-sum's exactness.
template <typename T> __device__ __forceinline__ void comp_add(T &hi, T &lo, T d) {
    const T s = add_rn(hi, d);
    const T bb = sub_rn(s, hi);
    const T err = add_rn(sub_rn(hi, sub_rn(s, bb)), sub_rn(d, bb));
    const T l = add_rn(lo, err);
    const T h = add_rn(s, l);
    lo = sub_rn(l, sub_rn(h, s));
    hi = h;
}
// Two independent compensated adds, (h0, l0) += d0 and (h1, l1) += d1 (the real and imaginary
// parts of one entry, or two momentum components).  With LQ_PAIRED_ADD (the default) the FP32 form
// runs both lanes through the paired FP32 adds of sm_100 and later (__fadd2_rn), each lane rounding
// exactly as comp_add rounds it: bitwise the same results, 12 us less per k_md launch at 32^4.
#ifndef LQ_PAIRED_ADD
#define LQ_PAIRED_ADD 1
#endif
template <typename T> __device__ __forceinline__ void comp_add2(T &h0, T &h1, T &l0, T &l1, T d0, T d1) {
    comp_add(h0, l0, d0);
    comp_add(h1, l1, d1);
}
#if LQ_PAIRED_ADD
__device__ __forceinline__ float2 neg2(float2 x) { return make_float2(-x.x, -x.y); }
template <>
__device__ __forceinline__ void comp_add2<float>(float &h0, float &h1, float &l0, float &l1, float d0, float d1) {
    const float2 hi = make_float2(h0, h1), lo = make_float2(l0, l1), d = make_float2(d0, d1);
    const float2 s = __fadd2_rn(hi, d);
    const float2 bb = __fadd2_rn(s, neg2(hi));
    const float2 err = __fadd2_rn(__fadd2_rn(hi, neg2(__fadd2_rn(s, neg2(bb)))), __fadd2_rn(d, neg2(bb)));
    const float2 l = __fadd2_rn(lo, err);
    const float2 h = __fadd2_rn(s, l);
    const float2 nl = __fadd2_rn(l, neg2(__fadd2_rn(h, neg2(s))));
    h0 = h.x;
    h1 = h.y;
    l0 = nl.x;
    l1 = nl.y;
}
#endif
// split a double into a pair of T (exact for T = double with lo = 0)
template <typename T> __device__ __forceinline__ void split(double x, T &hi, T &lo) {
    hi = (T)x;
    lo = (T)(x - (double)hi);
}

// ------------------------------------------------------------------ block reductions
// Fixed-shape warp-shuffle + shared-memory tree: deterministic for a given launch shape.
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double *__restrict__ out, uint32_t slot,
                                                   uint32_t nslots) {
    __shared__ double red[32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) red[warp][i] = v[i];
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double x = (lane < nw) ? red[lane][i] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) out[(size_t)i * nslots + slot] = x;
        }
    }
}

// Sum NV rows of `n` partials each, in a fixed order, into out[0..NV).  One block of 1024.
template <int NV>
__global__ void __launch_bounds__(1024) k_finalize(const double *__restrict__ partial, uint32_t n, double *out) {
    double v[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double s = 0.0;
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) s += partial[(size_t)i * n + k];
        v[i] = s;
    }
    block_reduce_store<NV>(v, out, 0, 1);
}

// ------------------------------------------------------------------ gauge force
// Staple sum of link (x, mu) in the reference's order of directions [+0,-0,+1,-1,...]
// skipping +-mu (procedural_macro/src/lib.rs:53-83, src/simulation/state.rs:1428-1437):
//   +nu : U_nu(x+mu) U_mu(x+nu)^dag U_nu(x)^dag            = S_mu,nu(x)^dag
//   -nu : U_nu(x+mu-nu)^dag U_mu(x-nu)^dag U_nu(x-nu)      = S_mu,-nu(x)^dag
template <int D, typename T>
__device__ __forceinline__ void staple_sum(const V2<T> *__restrict__ U, const Geo<D> &g, uint32_t site,
                                           const uint32_t *c, int mu, mat3<T> &sig) {
    const uint32_t xpmu = fwd(g, site, c[mu], mu);
    mat_zero(sig);
#pragma unroll
    for (int nu = 0; nu < D; ++nu) {
        if (nu == mu) continue;
        {
            mat3<T> a, b, t;
            load_link<T>(U, tix(xpmu, D * 9, nu * 9), a);
            load_link<T>(U, tix(fwd(g, site, c[nu], nu), D * 9, mu * 9), b);
            mul_na(a, b, t);
            load_link<T>(U, tix(site, D * 9, nu * 9), a);
            mul_na_acc(t, a, sig);
        }
        {
            mat3<T> a, b, w;
            const uint32_t xmnu = bwd(g, site, c[nu], nu);
            load_link<T>(U, tix(xmnu, D * 9, mu * 9), a);
            load_link<T>(U, tix(bwd(g, xpmu, c[nu], nu), D * 9, nu * 9), b);
            mul_nn(a, b, w);
            load_link<T>(U, tix(xmnu, D * 9, nu * 9), a);
            mul_an_acc(w, a, sig);
        }
    }
}

enum : int { MD_KICK = 1, MD_DRIFT = 2, MD_DRIFT_OLD_E = 4, MD_EXP = 8, MD_REUNIT = 16 };

// k_md: one thread per link.  Blocks are ordered with mu fastest (blockIdx.x = site_block*D + mu)
// so the D directions of a block of sites run together and the neighbour links they share
// stay in L2.
//  KICK : F^a = Im Tr(T^a U_mu(x) Sigma(x)) (derivative_e, src/simulation/state.rs:1420-1448);
//         e += k1 * F (when k1 != 0), then e += k2 * F, with k = h * c_e / size,
//         c_e = -sqrt(2/C_A).  Two separate adds keep the reference's rounding of a step end
//         followed by the next step's start (src/integrator/symplectic_euler_rayon.rs:222-252).
//         E is read from Ein and written to Eout (the same buffer for an in-place update).
//  DRIFT: U' = U + drift * i (E U), drift = dt sqrt(2 C_A) / size
//         (derivative_u + integrate_link, src/simulation/state.rs:1407-1417,
//          src/integrator/mod.rs:216-233), with E after the kick or, with DRIFT_OLD_E,
//         before it (integrate_sync_sync integrates both fields from the old state).
//         With EXP the link moves on the group instead: U' = exp(i drift E) U, the
//         exponential by su3_exp_i's Cayley-Hamilton recursion; REUNIT then applies
//         orthonormalize_matrix to the result (in double, from hi + lo).
// md_update applies the kick (with the staple sum sig) and the drift to link (site, mu), reading
// the link and its momenta from Uin / Ein (lo halves at ulo / elo elements further).
// md_kick_drift: md_update's kick and drift of link (site, mu) from its force coefficients
// f^a = Im Tr(T^a U_mu(x) Sigma_mu(x)) and the link u = U_mu(x) itself.
template <int D, typename T, bool COMP, int MODE>
__device__ __forceinline__ void md_kick_drift(const T (&f)[8], mat3<T> &u, const V2<T> *__restrict__ Uin, const T *Ein,
                                              V2<T> *__restrict__ Uout, T *Eout, bool copy_e, uint32_t site, int mu,
                                              T k1, T k2, T drift, size_t ulo, size_t elo);

template <int D, typename T, bool COMP, int MODE>
__device__ __forceinline__ void md_update(const mat3<T> &sig, const V2<T> *__restrict__ Uin, const T *Ein,
                                          V2<T> *__restrict__ Uout, T *Eout, bool copy_e, uint32_t site, int mu,
                                          T k1, T k2, T drift, size_t ulo, size_t elo) {
    mat3<T> u;
    load_link<T>(Uin, tix(site, D * 9, mu * 9), u);
    T f[8];
    if (MODE & MD_KICK) im_tr_generators_of_product(u, sig, f);
    md_kick_drift<D, T, COMP, MODE>(f, u, Uin, Ein, Uout, Eout, copy_e, site, mu, k1, k2, drift, ulo, elo);
}

template <int D, typename T, bool COMP, int MODE>
__device__ __forceinline__ void md_kick_drift(const T (&f)[8], mat3<T> &u, const V2<T> *__restrict__ Uin, const T *Ein,
                                              V2<T> *__restrict__ Uout, T *Eout, bool copy_e, uint32_t site, int mu,
                                              T k1, T k2, T drift, size_t ulo, size_t elo) {
    const size_t ui = tix(site, D * 9, mu * 9), ei = tix(site, D * 8, mu * 8);
    T e[8], el[8], e_old[8];
    load_efield<T>(Ein, ei, e);
    if (COMP) load_efield<T>(Ein + elo, ei, el);
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        if (!COMP) el[a] = T(0);
        e_old[a] = e[a];
    }
    if (MODE & MD_KICK) {
        if (COMP) {
            // compensated storage: one exact-sum update with both half-kicks (the separate
            // adds of the FP64 form only reproduce the reference's FP64 rounding)
            const T k = k1 + k2;
#pragma unroll
            for (int a = 0; a < 8; a += 2) comp_add2(e[a], e[a + 1], el[a], el[a + 1], k * f[a], k * f[a + 1]);
            store_efield<T>(Eout + elo, ei, el);
        } else {
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                if (k1 != T(0)) e[a] = fma(k1, f[a], e[a]);
                e[a] = fma(k2, f[a], e[a]);
            }
        }
        store_efield<T>(Eout, ei, e);
    } else if (copy_e) {
        store_efield<T>(Eout, ei, e);
        if (COMP) store_efield<T>(Eout + elo, ei, el);
    }
    if (MODE & MD_DRIFT) {
        const T *ed = (MODE & MD_DRIFT_OLD_E) ? e_old : e;
        // w: the increment U' - U
        mat3<T> w;
        if (MODE & MD_EXP) {
            T v[8];
#pragma unroll
            for (int a = 0; a < 8; ++a) v[a] = drift * ed[a];
            mat3<T> r;
            su3_exp_i_minus_one<T>(v, r);
            mul_nn(r, u, w);
        } else {
            mat3<T> x;
            adj_mul<T>(ed, u, x);
#pragma unroll
            for (int k = 0; k < 9; ++k) w.e[k] = cmk(-drift * x.e[k].im, drift * x.e[k].re);
        }
        mat3<T> ul;
        if (COMP) load_link<T>(Uin + ulo, ui, ul);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            if (COMP) {
                comp_add2(u.e[k].re, u.e[k].im, ul.e[k].re, ul.e[k].im, w.e[k].re, w.e[k].im);
            } else {
                u.e[k].re += w.e[k].re;
                u.e[k].im += w.e[k].im;
            }
        }
        if (MODE & MD_REUNIT) {
            double re[9], im[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                re[k] = (double)u.e[k].re + (COMP ? (double)ul.e[k].re : 0.0);
                im[k] = (double)u.e[k].im + (COMP ? (double)ul.e[k].im : 0.0);
            }
            orthonormalize_d(re, im);
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                T lr, li;
                split(re[k], u.e[k].re, lr);
                split(im[k], u.e[k].im, li);
                if (COMP) ul.e[k] = cmk(lr, li);
            }
        }
        if (COMP) store_link<T>(Uout + ulo, ui, ul);
        store_link<T>(Uout, ui, u);
    }
}
// md_link computes link (site, mu): the staple sum first, then the link and momenta of (x, mu)
// are loaded (after it, so they do not occupy registers while the neighbour links are in
// flight); ulo / elo: distance in elements from a hi array to its lo array.
template <int D, typename T, bool COMP, int MODE>
__device__ __forceinline__ void md_link(const V2<T> *__restrict__ Uin, V2<T> *__restrict__ Uout, const T *Ein,
                                        T *Eout, const Geo<D> &g, uint32_t site, int mu, T k1, T k2, T drift,
                                        size_t ulo, size_t elo) {
    mat3<T> sig;
    if (MODE & MD_KICK) {
        uint32_t c[D];
        site_coords(g, site, c);
        staple_sum<D, T>(Uin, g, site, c, mu, sig);
    }
    md_update<D, T, COMP, MODE>(sig, Uin, Ein, Uout, Eout, Eout != Ein, site, mu, k1, k2, drift, ulo, elo);
}

template <int D, typename T, bool COMP, int MODE>
__global__ void __launch_bounds__(128, MinBlocks<T>::md) k_md(const V2<T> *__restrict__ Uin, V2<T> *__restrict__ Uout, const T *Ein, T *Eout,
                                  Geo<D> g, T k1, T k2, T drift) {
    const uint32_t site = (blockIdx.x / D) * blockDim.x + threadIdx.x;
    const int mu = blockIdx.x % D;
    const size_t nt = tiles_of(g.V);
    const size_t ulo = nt * D * 9 * kTile, elo = nt * D * 8 * kTile;
    if (site >= g.V) return;
    md_link<D, T, COMP, MODE>(Uin, Uout, Ein, Eout, g, site, mu, k1, k2, drift, ulo, elo);
}

// k_md_site: the MD step with one thread per site and its D links, the plaquette products shared
// between the links that need them.  For the links (x, mu) and (x, nu) of one site, the +nu staple of
// the first and the +mu staple of the second close the same plaquette P_mu,nu(x) =
// U_mu(x) U_nu(x+mu) U_mu(x+nu)^dag U_nu(x)^dag: U_mu(x) S+_mu,nu(x) = P and U_nu(x) S+_nu,mu(x) =
// P^dag, so Im Tr(T^a .) of one product serves both links with opposite signs.  Per site the forward
// staples then cost D(D-1)/2 plaquettes (two products and one projected product each) instead of
// D(D-1) staples of two products each: 1964 instructions per link against 2200 for k_md (mixed, D = 4,
// ncu).  The backward staples keep staple_sum's products.  Each link's force
// is complete once the planes (mu, nu > mu) and (nu < mu, mu) and its backward staples are summed,
// and that link is kicked and drifted by md_update's arithmetic before the next direction.  The
// force is summed per plaquette rather than as one staple matrix, so the results differ from k_md's
// by rounding (the FP64 form's parity with the reference is unchanged at 1e-12).
template <int D, typename T, bool COMP, int MODE>
__device__ __forceinline__ void md_site(const V2<T> *__restrict__ Uin, V2<T> *__restrict__ Uout, const T *Ein, T *Eout,
                                        const Geo<D> &g, uint32_t site, T k1, T k2, T drift, size_t ulo, size_t elo,
                                        T (&fs)[(D - 1) * 8][kMdSiteBlock], unsigned t) {
    static_assert(MODE & MD_KICK, "the site kernel computes the force");
    uint32_t c[D];
    site_coords(g, site, c);
#pragma unroll
    for (int a = 0; a < (D - 1) * 8; ++a) fs[a][t] = T(0);
    // one direction at a time: with the directions unrolled the compiler spills (kilobytes of local
    // memory in the FP64 and several FP32 modes)
#pragma unroll 1
    for (int mu = 0; mu < D; ++mu) {
#if LQ_MD_PREFETCH
        // the update's own-link data (momenta hi and lo, the link's lo half) are read once, after the
        // force: ask L2 for them now, so that their DRAM latency passes under the force's products
        {
            const size_t ui = tix(site, D * 9, mu * 9), ei = tix(site, D * 8, mu * 8);
            constexpr int W = 16 / (int)sizeof(T); // reals per 16-byte momentum vector (load_efield)
            const size_t lane = ei & 31;
            const T *eq = Ein + (ei - lane) + lane * W;
#pragma unroll
            for (int j = 0; j < 8 / W; ++j) {
                asm volatile("prefetch.global.L2 [%0];" ::"l"(eq + j * W * kTile));
                if (COMP) asm volatile("prefetch.global.L2 [%0];" ::"l"(eq + elo + j * W * kTile));
            }
            if (COMP)
#pragma unroll
                for (int k = 0; k < 9; ++k) asm volatile("prefetch.global.L2 [%0];" ::"l"(Uin + ulo + ui + k * kTile));
        }
#endif
        const uint32_t xpmu = fwd(g, site, c[mu], mu);
        mat3<T> umu;
        load_link<T>(Uin, tix(site, D * 9, mu * 9), umu);
        T f[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) f[a] = mu == 0 ? T(0) : fs[(mu - 1) * 8 + a][t];
        // forward plaquettes of the planes (mu, nu > mu): P = U_mu(x) U_nu(x+mu) U_mu(x+nu)^dag U_nu(x)^dag
#pragma unroll
        for (int nu = mu + 1; nu < D; ++nu) {
            mat3<T> p, q, A;
            load_link<T>(Uin, tix(xpmu, D * 9, nu * 9), q);
            mul_nn(umu, q, A);
            load_link<T>(Uin, tix(fwd(g, site, c[nu], nu), D * 9, mu * 9), q);
            mul_na(A, q, p);
            load_link<T>(Uin, tix(site, D * 9, nu * 9), q);
            T pf[8];
            im_tr_generators_of_product_na(p, q, pf);
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                f[a] += pf[a];
                fs[(nu - 1) * 8 + a][t] -= pf[a];
            }
        }
        // backward staples of (x, mu): U_nu(x+mu-nu)^dag U_mu(x-nu)^dag U_nu(x-nu)
        mat3<T> sig;
        mat_zero(sig);
#pragma unroll
        for (int nu = 0; nu < D; ++nu) {
            if (nu == mu) continue;
            mat3<T> a, b, w;
            const uint32_t xmnu = bwd(g, site, c[nu], nu);
            load_link<T>(Uin, tix(xmnu, D * 9, mu * 9), a);
            load_link<T>(Uin, tix(bwd(g, xpmu, c[nu], nu), D * 9, nu * 9), b);
            mul_nn(a, b, w);
            load_link<T>(Uin, tix(xmnu, D * 9, nu * 9), a);
            mul_an_acc(w, a, sig);
        }
        T fb[8];
        im_tr_generators_of_product(umu, sig, fb);
#pragma unroll
        for (int a = 0; a < 8; ++a) f[a] += fb[a];
        md_kick_drift<D, T, COMP, MODE>(f, umu, Uin, Ein, Uout, Eout, Eout != Ein, site, mu, k1, k2, drift, ulo, elo);
    }
}

template <int D, typename T, bool COMP, int MODE>
__global__ void __launch_bounds__(kMdSiteBlock, MinBlocks<T>::md_site)
    k_md_site(const V2<T> *__restrict__ Uin, V2<T> *__restrict__ Uout, const T *Ein, T *Eout, Geo<D> g, T k1, T k2,
              T drift, BlockOrder bo) {
    // the parts of later directions' forces from the planes (mu, nu > mu), one column per thread
    __shared__ T fs[(D - 1) * 8][kMdSiteBlock];
    const uint32_t site = block_at(bo, blockIdx.x) * blockDim.x + threadIdx.x;
    if (site >= g.V) return;
    const size_t nt = tiles_of(g.V);
    md_site<D, T, COMP, MODE>(Uin, Uout, Ein, Eout, g, site, k1, k2, drift, nt * D * 9 * kTile, nt * D * 8 * kTile, fs,
                              threadIdx.x);
}

// U <- exp(i angle T^a) U for one link (finite-difference probes of the action)
template <int D, typename T, bool COMP>
__global__ void k_link_rotate(V2<T> *__restrict__ U, uint32_t V, uint32_t site, int mu, int a, T angle) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const size_t ui = tix(site, D * 9, mu * 9), ulo = (size_t)tiles_of(V) * D * 9 * kTile;
    T v[8];
#pragma unroll
    for (int b = 0; b < 8; ++b) v[b] = (b == a) ? angle : T(0);
    mat3<T> u, ul, r, w;
    load_link<T>(U, ui, u);
    if (COMP) load_link<T>(U + ulo, ui, ul);
    su3_exp_i_minus_one<T>(v, r);
    mul_nn(r, u, w);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        if (COMP) {
            comp_add(u.e[k].re, ul.e[k].re, w.e[k].re);
            comp_add(u.e[k].im, ul.e[k].im, w.e[k].im);
        } else {
            u.e[k].re += w.e[k].re;
            u.e[k].im += w.e[k].im;
        }
    }
    store_link<T>(U, ui, u);
    if (COMP) store_link<T>(U + ulo, ui, ul);
}

// ------------------------------------------------------------------ Gauss law
// G(x) is Hermitian; it is stored as 9 reals per site: the real diagonal and the upper
// off-diagonal entries, G[c*V + site] with c = (G00, G11, G22, Re G01, Im G01, Re G02,
// Im G02, Re G12, Im G12).  Links drift off SU(3) under the first-order link update, so
// U^dag E U acquires a small trace; keeping the full Hermitian G (not only its su(3)
// projection) follows the reference, whose G enters the projection step as a matrix.
template <typename T> __device__ __forceinline__ void herm_load(const T *__restrict__ G, uint32_t site, mat3<T> &m) {
    const T *p = G + tix(site, 9, 0);
    const T d0 = p[0], d1 = p[kTile], d2 = p[2 * kTile];
    const T r01 = p[3 * kTile], i01 = p[4 * kTile];
    const T r02 = p[5 * kTile], i02 = p[6 * kTile];
    const T r12 = p[7 * kTile], i12 = p[8 * kTile];
    m.e[0] = cmk(d0, T(0));
    m.e[4] = cmk(d1, T(0));
    m.e[8] = cmk(d2, T(0));
    m.e[1] = cmk(r01, i01);
    m.e[3] = cmk(r01, -i01);
    m.e[2] = cmk(r02, i02);
    m.e[6] = cmk(r02, -i02);
    m.e[5] = cmk(r12, i12);
    m.e[7] = cmk(r12, -i12);
}
template <typename T> __device__ __forceinline__ void herm_store(T *__restrict__ G, uint32_t site, const mat3<T> &m) {
    T *p = G + tix(site, 9, 0);
    p[0] = m.e[0].re;
    p[kTile] = m.e[4].re;
    p[2 * kTile] = m.e[8].re;
    p[3 * kTile] = m.e[1].re;
    p[4 * kTile] = m.e[1].im;
    p[5 * kTile] = m.e[2].re;
    p[6 * kTile] = m.e[2].im;
    p[7 * kTile] = m.e[5].re;
    p[8 * kTile] = m.e[5].im;
}

// G(x) = sum_mu [E_mu(x) - U_mu(x-mu)^dag E_mu(x-mu) U_mu(x-mu)]  (EField::gauss,
// src/field.rs:1174-1195); the per-site residual |Tr((sum_a T^a) G(x))| = |sum_a g^a| / 2,
// g^a = 2 Re Tr(T^a G) (gauss_sum_div, src/field.rs:1199-1220), is reduced into one
// partial per block.  Reads hi parts only.
template <int D, typename T>
__device__ __forceinline__ double gauss_site(const V2<T> *__restrict__ U, const T *__restrict__ E, T *__restrict__ G,
                                             const Geo<D> &g, uint32_t site) {
    {
        uint32_t c[D];
        site_coords(g, site, c);
        mat3<T> gs;
        mat_zero(gs);
#pragma unroll
        for (int mu = 0; mu < D; ++mu) {
            const uint32_t xm = bwd(g, site, c[mu], mu);
            const size_t ex = tix(site, D * 8, mu * 8), emi = tix(xm, D * 8, mu * 8);
            T ex_c[8], em_c[8];
            load_efield<T>(E, ex, ex_c);
            load_efield<T>(E, emi, em_c);
            mat3<T> u, ex_m, t, w;
            load_link<T>(U, tix(xm, D * 9, mu * 9), u);
            adjoint_to_matrix<T>(ex_c, ex_m);
            adj_mul<T>(em_c, u, t);
            mul_an_herm(u, t, w); // U^dag E U is Hermitian
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                gs.e[k].re += ex_m.e[k].re - w.e[k].re;
                gs.e[k].im += ex_m.e[k].im - w.e[k].im;
            }
        }
        herm_store(G, site, gs);
        T gc[8];
        two_re_tr_generators(gs, gc);
        T s = T(0);
#pragma unroll
        for (int a = 0; a < 8; ++a) s += gc[a];
        return (double)(fabs(s) * T(0.5));
    }
}
template <int D, typename T>
__global__ void __launch_bounds__(256) k_gauss(const V2<T> *__restrict__ U, const T *__restrict__ E,
                                               T *__restrict__ G, Geo<D> g, double *__restrict__ partial) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    double r[1] = {0.0};
    if (site < g.V) r[0] = gauss_site<D, T>(U, E, G, g, site);
    block_reduce_store<1>(r, partial, blockIdx.x, gridDim.x);
}

// One projection step on link (x, mu) (EField::project_to_gauss_step, src/field.rs:1301-1337):
//   e'^a = 2 Re Tr(T^a [(u G(x) u^dag G(x+mu) - G(x)) K + T^a e^a]),  K = 0.12
//        = e^a + K (2 Re Tr(T^a u G(x) u^dag G(x+mu)) - 2 Re Tr(T^a G(x)))
// with u = U_mu(x).  One function serves both call sites of k_gauss_sweep so that the
// recomputed update of a neighbour's link is the same arithmetic as its owner's.
template <typename T, bool COMP>
__device__ __forceinline__ void projection_step(const mat3<T> &u, const mat3<T> &gx, const T *gxc, const mat3<T> &gp,
                                                T *e, T *el) {
    mat3<T> t1, t2;
    mul_nh(u, gx, t1);      // G(x) Hermitian
    mul_na_herm(t1, u, t2); // u G(x) u^dag is Hermitian
    T xc[8];
    two_re_tr_generators_of_hermitian_product(t2, gp, xc);
    const T K = T(0.12);
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        if (COMP) comp_add(e[a], el[a], K * (xc[a] - gxc[a]));
        else e[a] = fma(K, xc[a] - gxc[a], e[a]);
    }
}

// ---- the FP64 projection in the adjoint representation ----
// The projection changes E only: its links are fixed.  So the maps X -> U X U^dag and
// X -> U^dag X U of every link on Hermitian 3x3 matrices are formed once per projection
// (k_adjoint_links), and every parallel transport in the sweeps becomes a real 9x9
// matrix-vector product instead of two complex 3x3 products.  A Hermitian X is held as its 9
// components x^a = 2 Re Tr(T^a X) (a < 8) and x^8 = Tr X, X = sum x^a T^a + (x^8 / 3) 1.  The
// trace is carried because the links are not exactly unitary: the leap-frog's first-order link
// update leaves |U U^dag - 1| ~ 1e-8 after a trajectory, and the reference transports with the
// full matrices, so U^dag E U has a trace and G(x) with it.  The two maps share one table per link:
//   R_ab = 2 Re Tr(T^a U T^b U^dag)      (U X U^dag: R;  U^dag X U: R^T, on the generator block)
//   A_a = 2 Re Tr(T^a U U^dag),  B_a = 2 Re Tr(T^a U^dag U),  t = Tr(U U^dag)
//   U X U^dag:  y^a = R_ab x^b + A_a x^8 / 3,   y^8 = B_b x^b / 2 + t x^8 / 3
//   U^dag X U:  y^a = R_ba x^b + B_a x^8 / 3,   y^8 = A_b x^b / 2 + t x^8 / 3
// The arithmetic is that of the matrix-form step (projection_step) and Gauss law (k_gauss) up to
// rounding: the FP64 state's projection, bound by its FP64 multiply-add rate.
//
// Layout of the table: the kAdjReals reals of the link (site, mu) fill planes mu*kAdjReals ..
// of a tile (tix(site, D * kAdjReals, mu * kAdjReals)): R row-major, A, B, t and one pad, packed in
// double2 pairs like the momenta (a thread moves a row of R with four 128-bit accesses).  G(x):
// kGaussReals planes per site (the 9 components and one pad), tix(site, kGaussReals, 0), packed the
// same way.
constexpr int kAdjReals = 82;
constexpr int kAdjA = 64, kAdjB = 72, kAdjT = 80;
constexpr int kGaussReals = 10;
template <int N>
__device__ __forceinline__ void load_packed(const double *__restrict__ A, size_t idx, int first, double *v) {
    const size_t lane = idx & 31;
    const double2 *q = reinterpret_cast<const double2 *>(A + (idx - lane)) + lane;
#pragma unroll
    for (int j = 0; j < N / 2; ++j) {
        const double2 x = q[(first / 2 + j) * kTile];
        v[2 * j] = x.x;
        v[2 * j + 1] = x.y;
    }
}
template <int N>
__device__ __forceinline__ void store_packed(double *__restrict__ A, size_t idx, int first, const double *v) {
    const size_t lane = idx & 31;
    double2 *q = reinterpret_cast<double2 *>(A + (idx - lane)) + lane;
#pragma unroll
    for (int j = 0; j < N / 2; ++j) q[(first / 2 + j) * kTile] = make_double2(v[2 * j], v[2 * j + 1]);
}

// the transport table of every link, one thread per link (directions fastest in the block order).  Row a of R holds the generator components of Q^a = U^dag T^a U, whose entries are
// sums of P^{rc}_ij = conj(U_ri) U_cj over the nonzero entries (r, c) of T^a (adjoint_to_matrix's
// Gell-Mann basis): with S = P^{rc} + P^{cr} and A = P^{cr} - P^{rc},
//   (r, c) = (0, 1): Q^0 = S / 2, Q^1 = i A / 2;  (0, 2): Q^3, Q^4;  (1, 2): Q^5, Q^6 likewise;
//   Q^2 = (P^{00} - P^{11}) / 2,  Q^7 = (P^{00} + P^{11} - 2 P^{22}) / (2 sqrt(3)).
// Column b of R is 2 Re Tr(T^b Q^a): 2 Re Q_01, -2 Im Q_01, Q_00 - Q_11, 2 Re Q_02, -2 Im Q_02,
// 2 Re Q_12, -2 Im Q_12, (Q_00 + Q_11 - 2 Q_22) / sqrt(3) (Q Hermitian).
template <int D, typename T>
__global__ void __launch_bounds__(128) k_adjoint_links(const V2<T> *__restrict__ U, T *__restrict__ R, Geo<D> g) {
    static_assert(sizeof(T) == 8, "the adjoint projection is the FP64 state's");
    const uint32_t site = (blockIdx.x / D) * blockDim.x + threadIdx.x;
    const int mu = blockIdx.x % D;
    if (site >= g.V) return;
    mat3<T> u;
    load_link<T>(U, tix(site, D * 9, mu * 9), u);
    const size_t ri = tix(site, D * kAdjReals, mu * kAdjReals);
    auto P = [&](int r, int i, int c, int j) { // conj(U_ri) U_cj
        const cpx<T> x = u.e[r * 3 + i], y = u.e[c * 3 + j];
        return cmk(fma(x.re, y.re, x.im * y.im), fma(x.re, y.im, -x.im * y.re));
    };
    const T r3 = T(2.0 * kOneOver2Sqrt3); // 1/sqrt(3)
    T Rm[8][8];
    // off-diagonal entries (i, j) of every Q^a, stored as R columns c0 = 2 Re Q_ij, c0 + 1 = -2 Im Q_ij
    // (a = P^{rc}, b = P^{cr}: Q^{g} = (a + b) / 2, Q^{g+1} = i (b - a) / 2)
    auto offdiag = [&](int i, int j, int c0) {
        const int rc[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        const int gs[3] = {0, 3, 5};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const cpx<T> a = P(rc[k][0], i, rc[k][1], j), b = P(rc[k][1], i, rc[k][0], j);
            Rm[gs[k]][c0] = a.re + b.re;
            Rm[gs[k]][c0 + 1] = -(a.im + b.im);
            Rm[gs[k] + 1][c0] = a.im - b.im;
            Rm[gs[k] + 1][c0 + 1] = a.re - b.re;
        }
        const cpx<T> p00 = P(0, i, 0, j), p11 = P(1, i, 1, j), p22 = P(2, i, 2, j);
        Rm[2][c0] = p00.re - p11.re;
        Rm[2][c0 + 1] = p11.im - p00.im;
        Rm[7][c0] = r3 * fma(T(-2), p22.re, p00.re + p11.re);
        Rm[7][c0 + 1] = -r3 * fma(T(-2), p22.im, p00.im + p11.im);
    };
    offdiag(0, 1, 0);
    offdiag(0, 2, 3);
    offdiag(1, 2, 5);
    // the real diagonal entries Q^a_ii (P^{cr}_ii = conj(P^{rc}_ii)): columns 2 (Q_00 - Q_11) and 7
    // ((Q_00 + Q_11 - 2 Q_22) / sqrt(3))
    T d[3][8];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const T p00 = P(0, i, 0, i).re, p11 = P(1, i, 1, i).re, p22 = P(2, i, 2, i).re;
        const int rc[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        const int gs[3] = {0, 3, 5};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const cpx<T> a = P(rc[k][0], i, rc[k][1], i);
            d[i][gs[k]] = a.re; // (a + conj(a)) / 2
            d[i][gs[k] + 1] = a.im; // i (conj(a) - a) / 2
        }
        d[i][2] = T(0.5) * (p00 - p11);
        d[i][7] = T(kOneOver2Sqrt3) * fma(T(-2), p22, p00 + p11);
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        Rm[a][2] = d[0][a] - d[1][a];
        Rm[a][7] = r3 * fma(T(-2), d[2][a], d[0][a] + d[1][a]);
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) store_packed<8>(R, ri, a * 8, Rm[a]);
    mat3<T> w;
    T v[8];
    mul_na(u, u, w); // U U^dag
    two_re_tr_generators(w, v);
    store_packed<8>(R, ri, kAdjA, v);
    const T tr[2] = {w.e[0].re + w.e[4].re + w.e[8].re, T(0)};
    mul_an(u, u, w); // U^dag U
    two_re_tr_generators(w, v);
    store_packed<8>(R, ri, kAdjB, v);
    store_packed<2>(R, ri, kAdjT, tr);
}

// G(x) (9 components) and the residual partials (k_gauss's Gauss law), E traceless:
//   G(x) = sum_mu [E_mu(x) - U_mu(x-mu)^dag E_mu(x-mu) U_mu(x-mu)]
template <int D, typename T>
__global__ void __launch_bounds__(256) k_gauss_adj(const T *__restrict__ R, const T *__restrict__ E,
                                                   T *__restrict__ G, Geo<D> g, double *__restrict__ partial) {
    static_assert(sizeof(T) == 8, "the adjoint projection is the FP64 state's");
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    double res[1] = {0.0};
    if (site < g.V) {
        uint32_t c[D];
        site_coords(g, site, c);
        T gs[kGaussReals];
#pragma unroll
        for (int a = 0; a < kGaussReals; ++a) gs[a] = T(0);
#pragma unroll
        for (int mu = 0; mu < D; ++mu) {
            const uint32_t xm = bwd(g, site, c[mu], mu);
            T ex[8], em[8], av[8];
            load_efield<T>(E, tix(site, D * 8, mu * 8), ex);
            load_efield<T>(E, tix(xm, D * 8, mu * 8), em);
#pragma unroll
            for (int a = 0; a < 8; ++a) gs[a] += ex[a];
            const size_t ri = tix(xm, D * kAdjReals, mu * kAdjReals);
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                T row[8];
                load_packed<8>(R, ri, b * 8, row);
#pragma unroll
                for (int a = 0; a < 8; ++a) gs[a] = fma(-row[a], em[b], gs[a]);
            }
            load_packed<8>(R, ri, kAdjA, av);
            T tr = T(0);
#pragma unroll
            for (int b = 0; b < 8; ++b) tr = fma(av[b], em[b], tr);
            gs[8] = fma(T(-0.5), tr, gs[8]);
        }
        store_packed<kGaussReals>(G, tix(site, kGaussReals, 0), 0, gs);
        T sum = T(0);
#pragma unroll
        for (int a = 0; a < 8; ++a) sum += gs[a];
        res[0] = (double)(fabs(sum) * T(0.5));
    }
    block_reduce_store<1>(res, partial, blockIdx.x, gridDim.x);
}

// One projection step on every link from the components of G (projection_step's arithmetic):
//   e^a += 0.12 (2 Re Tr(T^a H G(x+mu)) - 2 Re Tr(T^a G(x))),  H = U G(x) U^dag
// with 2 Re Tr(T^a H P) = 2 Re Tr(T^a H0 P0) + h^8 p^a / 3 + p^8 h^a / 3 for H0, P0 the
// traceless parts; the factor 0.12 rides on the constants of each term.
template <int D, typename T>
__global__ void __launch_bounds__(128) k_gauss_step_adj(const T *__restrict__ R, T *__restrict__ E,
                                                        const T *__restrict__ G, Geo<D> g) {
    static_assert(sizeof(T) == 8, "the adjoint projection is the FP64 state's");
    const uint32_t site = (blockIdx.x / D) * blockDim.x + threadIdx.x;
    const int mu = blockIdx.x % D;
    if (site >= g.V) return;
    uint32_t c[D];
    site_coords(g, site, c);
    T gx[kGaussReals], gp[kGaussReals], h[8], e[8], v[8];
    load_packed<kGaussReals>(G, tix(site, kGaussReals, 0), 0, gx);
    load_packed<kGaussReals>(G, tix(fwd(g, site, c[mu], mu), kGaussReals, 0), 0, gp);
    const size_t ri = tix(site, D * kAdjReals, mu * kAdjReals);
    const T g8 = gx[8] * T(1.0 / 3.0);
    load_packed<8>(R, ri, kAdjA, v);
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        T row[8];
        load_packed<8>(R, ri, a * 8, row);
        T acc = v[a] * g8;
#pragma unroll
        for (int b = 0; b < 8; ++b) acc = fma(row[b], gx[b], acc);
        h[a] = acc;
    }
    T tr[2];
    load_packed<8>(R, ri, kAdjB, v);
    load_packed<2>(R, ri, kAdjT, tr);
    T h8 = T(0);
#pragma unroll
    for (int b = 0; b < 8; ++b) h8 = fma(v[b], gx[b], h8);
    h8 = fma(T(0.5), h8, tr[0] * g8);
    const T K = T(0.12);
    const T kh8 = K * (h8 * T(1.0 / 3.0)), kp8 = K * (gp[8] * T(1.0 / 3.0));
    const size_t ei = tix(site, D * 8, mu * 8);
    load_efield<T>(E, ei, e);
#pragma unroll
    for (int a = 0; a < 8; ++a) e[a] = fma(kp8, h[a], fma(kh8, gp[a], fma(-K, gx[a], e[a])));
    two_re_tr_generators_of_traceless_product(h, gp, K, e);
    store_efield<T>(E, ei, e);
}

// ---- the FP64 state's MD step in two launches ----
// k_md_plaq forms each plaquette's products once and hands the force on all four of its links: with
// a = U_mu(x), b = U_nu(x+mu), c = U_mu(x+nu), d = U_nu(x), A = a b, B = d c (mu < nu),
//   (x, mu) +Im Tr(T^a A B^dag)   and  (x, nu) -Im Tr(T^a A B^dag)   (the +nu / +mu staples, P = A B^dag)
//   (x+nu, mu)  Im Tr(T^a c A^dag d)                                   (its -nu staple b^dag a^dag d)
//   (x+mu, nu)  Im Tr(T^a b B^dag a)                                   (its -mu staple c^dag d^dag a)
// 4 products and 3 projections per plaquette, against 6 products and 2 projections (each a share of
// one staple-sum projection) when the backward staples are formed again by the sites that need them.
// The parts (twice their value: the projections' factor 1/2 is applied once, to the kick factors)
// land in the scratch array, D slots of 8 reals per link: slot 0 the forward part (the
// planes through the link's own site, summed in plane order), slot 1 + k the backward part from the
// k-th direction other than the link's; k_md_update sums the slots in that order and applies
// md_update's kick and drift.  FP64 only: the FP64 state is bound by its multiply-add rate, where
// the shared products turn into time, while the FP32 forms are bound by issue and latency and would
// pay the slots' extra traffic.  Scratch layout: tix(site, D * D * 8, mu * D * 8), packed double2
// pairs like the momenta.
template <int D> __device__ __forceinline__ int md_slot(int from, int link_dir) {
    return 1 + (from < link_dir ? from : from - 1);
}

template <int D, typename T>
__global__ void __launch_bounds__(128) k_md_plaq(const V2<T> *__restrict__ U, T *__restrict__ F, Geo<D> g) {
    static_assert(sizeof(T) == 8, "the split MD step is the FP64 state's");
    __shared__ T fs[D * 8][128]; // forward parts, one column per thread
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    if (site >= g.V) return;
    const unsigned t = threadIdx.x;
    uint32_t c[D];
    site_coords(g, site, c);
#pragma unroll
    for (int a = 0; a < D * 8; ++a) fs[a][t] = T(0);
#pragma unroll 1
    for (int mu = 0; mu < D - 1; ++mu) {
        const uint32_t xpmu = fwd(g, site, c[mu], mu);
#pragma unroll 1
        for (int nu = mu + 1; nu < D; ++nu) {
            const uint32_t xpnu = fwd(g, site, c[nu], nu);
            mat3<T> l, m, A, B, X;
            T f[8];
            load_link<T>(U, tix(site, D * 9, mu * 9), l);
            load_link<T>(U, tix(xpmu, D * 9, nu * 9), m);
            mul_nn(l, m, A); // a b
            load_link<T>(U, tix(site, D * 9, nu * 9), l);
            load_link<T>(U, tix(xpnu, D * 9, mu * 9), m);
            mul_nn(l, m, B); // d c
            im_tr_generators_of_product_na<T, false>(A, B, f);
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                fs[mu * 8 + a][t] += f[a];
                fs[nu * 8 + a][t] -= f[a];
            }
            mul_na(m, A, X); // c A^dag
            im_tr_generators_of_product<T, false>(X, l, f);
            store_packed<8>(F, tix(xpnu, D * D * 8, mu * D * 8), md_slot<D>(nu, mu) * 8, f);
            load_link<T>(U, tix(xpmu, D * 9, nu * 9), m);
            mul_na(m, B, X); // b B^dag
            load_link<T>(U, tix(site, D * 9, mu * 9), l);
            im_tr_generators_of_product<T, false>(X, l, f);
            store_packed<8>(F, tix(xpmu, D * D * 8, nu * D * 8), md_slot<D>(mu, nu) * 8, f);
        }
    }
#pragma unroll
    for (int mu = 0; mu < D; ++mu) {
        T f[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) f[a] = fs[mu * 8 + a][t];
        store_packed<8>(F, tix(site, D * D * 8, mu * D * 8), 0, f);
    }
}

template <int D, typename T, bool COMP, int MODE>
__global__ void __launch_bounds__(128) k_md_update(const V2<T> *__restrict__ Uin, V2<T> *__restrict__ Uout,
                                                   const T *Ein, T *Eout, const T *__restrict__ F, Geo<D> g, T k1,
                                                   T k2, T drift) {
    static_assert(sizeof(T) == 8, "the split MD step is the FP64 state's");
    static_assert(MODE & MD_KICK, "the force parts are summed for a kick");
    const uint32_t site = (blockIdx.x / D) * blockDim.x + threadIdx.x;
    const int mu = blockIdx.x % D;
    if (site >= g.V) return;
    const size_t nt = tiles_of(g.V);
    const size_t fi = tix(site, D * D * 8, mu * D * 8);
    T f[8], p[8];
    load_packed<8>(F, fi, 0, f);
#pragma unroll
    for (int k = 1; k < D; ++k) {
        load_packed<8>(F, fi, k * 8, p);
#pragma unroll
        for (int a = 0; a < 8; ++a) f[a] += p[a];
    }
    mat3<T> u;
    load_link<T>(Uin, tix(site, D * 9, mu * 9), u);
    // the parts are twice the force (k_md_plaq leaves the projections' factor 1/2 out): halving the
    // kick factors instead rounds the same
    md_kick_drift<D, T, COMP, MODE>(f, u, Uin, Ein, Uout, Eout, Eout != Ein, site, mu, T(0.5) * k1, T(0.5) * k2,
                                    drift, nt * D * 9 * kTile, nt * D * 8 * kTile);
}

// One projection sweep fused with the Gauss law of its result, one thread per site x:
//   E'_mu(x)    = step(U_mu(x),    G(x),    G(x+mu), E_mu(x))      written to Eout
//   E'_mu(x-mu) = step(U_mu(x-mu), G(x-mu), G(x),    E_mu(x-mu))   recomputed, not written
//   G'(x) = sum_mu [E'_mu(x) - U_mu(x-mu)^dag E'_mu(x-mu) U_mu(x-mu)]   written to Gout
// plus the residual partials of G'.  E and G are double-buffered (a thread reads its
// neighbours' old values while they are being replaced).  U is read once per sweep instead
// of twice (Gauss law, then step) and the sweep needs one launch instead of two.
template <int D, typename T, bool COMP, bool SHARE0 = false, bool SHARE1 = false>
__device__ __forceinline__ double sweep_site(const V2<T> *__restrict__ U, const T *__restrict__ Ein,
                                             T *__restrict__ Eout, const T *__restrict__ Gin, T *__restrict__ Gout,
                                             const Geo<D> &g, uint32_t site, size_t elo, T (*s1)[128] = nullptr,
                                             bool pf = false) {
    {
        uint32_t c[D];
        site_coords(g, site, c);
        // SHARE0 (the caller has checked that L divides 32 and every lane of a warp holds a site, so
        // the rows lie whole inside the warps): the step of link (x - 0, 0) is the own step of the
        // lane holding x - 0, taken by a shuffle instead of recomputed -- the same arithmetic on the
        // same inputs, so the same bits.  SHARE1 (L = 32 and every thread of a block a site, so the
        // block's four warps are four consecutive rows): warps 1..3 take the step of link
        // (x - 1, 1) from the warp before theirs through shared memory (s1, after a barrier every
        // thread of the block reaches); warp 0 recomputes it
        mat3<T> gx, gnew;
        if (pf) {
            // this site's momenta and its links U_mu(x), mu >= 1 (the step of direction 0 loads its link
            // at once), requested from L2 ahead of their loads
            constexpr int W = 16 / (int)sizeof(T); // reals per 16-byte momentum vector (load_efield)
#pragma unroll
            for (int mu = 0; mu < D; ++mu) {
                const size_t ei = tix(site, D * 8, mu * 8), lane = ei & 31;
                const T *eq = Ein + (ei - lane) + lane * W;
#pragma unroll
                for (int j = 0; j < 8 / W; ++j) asm volatile("prefetch.global.L2 [%0];" ::"l"(eq + j * W * kTile));
                if (mu > 0)
#pragma unroll
                    for (int k = 0; k < 9; ++k)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(U + tix(site, D * 9, mu * 9) + k * kTile));
            }
        }
        herm_load(Gin, site, gx);
        T gxc[8];
        two_re_tr_generators(gx, gxc);
        mat_zero(gnew);
#pragma unroll
        for (int mu = 0; mu < D; ++mu) {
            T e[8], el[8];
            {
                mat3<T> u, gp, em;
                load_link<T>(U, tix(site, D * 9, mu * 9), u);
                herm_load(Gin, fwd(g, site, c[mu], mu), gp);
                const size_t ei = tix(site, D * 8, mu * 8);
                load_efield<T>(Ein, ei, e);
                if (COMP) load_efield<T>(Ein + elo, ei, el);
                else
#pragma unroll
                    for (int a = 0; a < 8; ++a) el[a] = T(0);
                projection_step<T, COMP>(u, gx, gxc, gp, e, el);
                store_efield<T>(Eout, ei, e);
                if (COMP) store_efield<T>(Eout + elo, ei, el);
                if (SHARE1 && mu == 1) {
#pragma unroll
                    for (int a = 0; a < 8; ++a) s1[a][threadIdx.x] = e[a];
                    __syncthreads();
                }
                adjoint_to_matrix<T>(e, em);
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    gnew.e[k].re += em.e[k].re;
                    gnew.e[k].im += em.e[k].im;
                }
            }
            {
                const uint32_t xm = bwd(g, site, c[mu], mu);
                mat3<T> w, t, wm;
                load_link<T>(U, tix(xm, D * 9, mu * 9), w);
                if (!COMP && SHARE0 && mu == 0) {
                    const unsigned lane = site & (kTile - 1);
                    const unsigned src = c[0] > 0 ? lane - 1 : lane + g.L - 1;
#pragma unroll
                    for (int a = 0; a < 8; ++a) e[a] = __shfl_sync(0xffffffffu, e[a], src);
                } else if (!COMP && SHARE1 && mu == 1 && threadIdx.x >= kTile) {
#pragma unroll
                    for (int a = 0; a < 8; ++a) e[a] = s1[a][threadIdx.x - kTile];
                } else {
                    mat3<T> gm;
                    herm_load(Gin, xm, gm);
                    T gmc[8];
                    two_re_tr_generators(gm, gmc);
                    const size_t ei = tix(xm, D * 8, mu * 8);
                    load_efield<T>(Ein, ei, e);
                    if (COMP) load_efield<T>(Ein + elo, ei, el);
                    else
#pragma unroll
                        for (int a = 0; a < 8; ++a) el[a] = T(0);
                    projection_step<T, COMP>(w, gm, gmc, gx, e, el);
                }
                adj_mul<T>(e, w, t);
                mul_an_herm(w, t, wm); // U^dag E' U is Hermitian
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    gnew.e[k].re -= wm.e[k].re;
                    gnew.e[k].im -= wm.e[k].im;
                }
            }
        }
        herm_store(Gout, site, gnew);
        T gc[8];
        two_re_tr_generators(gnew, gc);
        T sum = T(0);
#pragma unroll
        for (int a = 0; a < 8; ++a) sum += gc[a];
        return (double)(fabs(sum) * T(0.5));
    }
}
template <int D, typename T, bool COMP, bool SHARE0 = false, bool SHARE1 = false>
__global__ void __launch_bounds__(128, MinBlocks<T>::sweep) k_gauss_sweep(const V2<T> *__restrict__ U, const T *__restrict__ Ein,
                                                     T *__restrict__ Eout, const T *__restrict__ Gin,
                                                     T *__restrict__ Gout, Geo<D> g, double *__restrict__ partial,
                                                     BlockOrder bo, int pf) {
    __shared__ T s1[SHARE1 ? 8 : 1][128];
    const uint32_t blk = block_at(bo, blockIdx.x); // the residual partial keeps its site-order slot
    const uint32_t site = blk * blockDim.x + threadIdx.x;
    double r[1] = {0.0};
    if (site < g.V)
        r[0] = sweep_site<D, T, COMP, SHARE0, SHARE1>(U, Ein, Eout, Gin, Gout, g, site,
                                                      (size_t)tiles_of(g.V) * D * 8 * kTile, s1, pf != 0);
    block_reduce_store<1>(r, partial, blk, gridDim.x);
}

// ------------------------------------------------------------------ plaquettes
// Per site, for mu < nu: P = U_mu(x) U_nu(x+mu) U_mu(x+nu)^dag U_nu(x)^dag
// (pij, src/field.rs:761-771), Tr P = Tr(A B^dag) with A = U_mu(x) U_nu(x+mu),
// B = U_nu(x) U_mu(x+nu).  Partials: [0] sum (1 - Re Tr P / 3) (hamiltonian_links,
// src/simulation/state.rs:821-849), [1] sum Re Tr P, [2] sum Im Tr P
// (average_trace_plaquette, src/field.rs:775-804).  The traces of one site accumulate in
// T (hi parts of compensated links) and every sum over sites in double.
template <int D, typename T>
__device__ __forceinline__ void plaquette_site(const V2<T> *__restrict__ U, const Geo<D> &g, uint32_t site,
                                               double (&v)[3]) {
    {
        uint32_t c[D];
        site_coords(g, site, c);
        T sre = T(0), sim = T(0), sh = T(0);
#pragma unroll
        for (int mu = 0; mu < D; ++mu) {
            const uint32_t xpmu = fwd(g, site, c[mu], mu);
#pragma unroll
            for (int nu = mu + 1; nu < D; ++nu) {
                mat3<T> p, q, A, B;
                load_link<T>(U, tix(site, D * 9, mu * 9), p);
                load_link<T>(U, tix(xpmu, D * 9, nu * 9), q);
                mul_nn(p, q, A);
                load_link<T>(U, tix(site, D * 9, nu * 9), p);
                load_link<T>(U, tix(fwd(g, site, c[nu], nu), D * 9, mu * 9), q);
                mul_nn(p, q, B);
                T re = T(0), im = T(0);
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    re = fma(A.e[k].re, B.e[k].re, re);
                    re = fma(A.e[k].im, B.e[k].im, re);
                    im = fma(A.e[k].im, B.e[k].re, im);
                    im = fma(-A.e[k].re, B.e[k].im, im);
                }
                sh += T(1) - re / T(3);
                sre += re;
                sim += im;
            }
        }
        v[0] = (double)sh;
        v[1] = (double)sre;
        v[2] = (double)sim;
    }
}
template <int D, typename T>
__global__ void __launch_bounds__(128) k_plaquette(const V2<T> *__restrict__ U, Geo<D> g,
                                                   double *__restrict__ partial) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    if (site < g.V) plaquette_site<D, T>(U, g, site, v);
    block_reduce_store<3>(v, partial, blockIdx.x, gridDim.x);
}

// Difference of the plaquette sums of two link fields, Re Tr[P(U') - P(U)] summed over
// every plaquette, evaluated without cancellation: with P = A B C^dag Dd^dag
// (A = U_mu(x), B = U_nu(x+mu), C = U_mu(x+nu), Dd = U_nu(x)) the exact telescoping
//   P' - P = dA B' C'^dag Dd'^dag + A dB C'^dag Dd'^dag + A B dC^dag Dd'^dag + A B C^dag dDd^dag
// needs only products with one difference factor, so FP32 products leave an error
// proportional to |dU|, not to |U|.  dU = (hi' - hi) + (lo' - lo) keeps the compensated part.
// Partial: sum Re Tr(P' - P) (Delta hamiltonian_links = -beta/3 times it).
template <int D, typename T, bool COMP>
__device__ __forceinline__ double plaquette_delta_site(const V2<T> *__restrict__ Uo, const V2<T> *__restrict__ Un,
                                                       const Geo<D> &g, uint32_t site, size_t ulo) {
    {
        uint32_t c[D];
        site_coords(g, site, c);
        auto load_pair = [&](int dir, uint32_t x, mat3<T> &old_hi, mat3<T> &new_hi, mat3<T> &diff) {
            const size_t i = tix(x, D * 9, dir * 9);
            load_link<T>(Uo, i, old_hi);
            load_link<T>(Un, i, new_hi);
            if (COMP) {
                mat3<T> ol, nl;
                load_link<T>(Uo + ulo, i, ol);
                load_link<T>(Un + ulo, i, nl);
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    diff.e[k].re = (new_hi.e[k].re - old_hi.e[k].re) + (nl.e[k].re - ol.e[k].re);
                    diff.e[k].im = (new_hi.e[k].im - old_hi.e[k].im) + (nl.e[k].im - ol.e[k].im);
                }
            } else {
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    diff.e[k].re = new_hi.e[k].re - old_hi.e[k].re;
                    diff.e[k].im = new_hi.e[k].im - old_hi.e[k].im;
                }
            }
        };
        // Re Tr(X Y) and Re Tr(X Y^dag)
        auto re_tr_nn = [](const mat3<T> &x, const mat3<T> &y) {
            T s = T(0);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    s = fma(x.e[i * 3 + k].re, y.e[k * 3 + i].re, s);
                    s = fma(-x.e[i * 3 + k].im, y.e[k * 3 + i].im, s);
                }
            return s;
        };
        auto re_tr_na = [](const mat3<T> &x, const mat3<T> &y) {
            T s = T(0);
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                s = fma(x.e[k].re, y.e[k].re, s);
                s = fma(x.e[k].im, y.e[k].im, s);
            }
            return s;
        };
        T acc = T(0);
#pragma unroll 1
        for (int mu = 0; mu < D; ++mu) {
            const uint32_t xpmu = fwd(g, site, c[mu], mu);
#pragma unroll 1
            for (int nu = mu + 1; nu < D; ++nu) {
                const uint32_t xpnu = fwd(g, site, c[nu], nu);
                // links: A = U_mu(x), B = U_nu(x+mu), C = U_mu(x+nu), Dd = U_nu(x); primes: new.
                // Evaluated in an order that keeps about four matrices live.
                mat3<T> q1, t, s1, x_old, x_new, dx, l1;
                T term = T(0);
                load_link<T>(Un, tix(site, D * 9, nu * 9), x_new); // Dd'
                load_link<T>(Un, tix(xpnu, D * 9, mu * 9), t);     // C'
                mul_nn(x_new, t, q1);                                  // Q1 = Dd' C'
                load_link<T>(Un, tix(xpmu, D * 9, nu * 9), t);     // B'
                mul_na(t, q1, s1);                                     // B' C'^dag Dd'^dag
                load_pair(mu, site, x_old, x_new, dx);                 // A, A', dA
                term += re_tr_nn(dx, s1);                              // Tr(dA B' C'^dag Dd'^dag)
                mul_an(q1, x_old, t);                                  // C'^dag Dd'^dag A
                mat3<T> a_old = x_old;
                load_pair(nu, xpmu, x_old, x_new, dx);                 // B, B', dB
                term += re_tr_nn(dx, t);                               // Tr(A dB C'^dag Dd'^dag)
                mul_nn(a_old, x_old, l1);                              // L1 = A B
                load_link<T>(Un, tix(site, D * 9, nu * 9), x_new); // Dd'
                mul_an(x_new, l1, t);                                  // Dd'^dag A B
                load_pair(mu, xpnu, x_old, x_new, dx);                 // C, C', dC
                term += re_tr_na(t, dx);                               // Tr(A B dC^dag Dd'^dag)
                mul_na(l1, x_old, t);                                  // A B C^dag
                load_pair(nu, site, x_old, x_new, dx);                 // Dd, Dd', dDd
                term += re_tr_na(t, dx);                               // Tr(A B C^dag dDd^dag)
                acc += term;
            }
        }
        return (double)acc;
    }
}
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128, (MinBlocksDelta<D, T>::value))
    k_plaquette_delta(const V2<T> *__restrict__ Uo, const V2<T> *__restrict__ Un, Geo<D> g, double *__restrict__ partial) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (site < g.V)
        v[0] = plaquette_delta_site<D, T, COMP>(Uo, Un, g, site, (size_t)tiles_of(g.V) * D * 9 * kTile);
    block_reduce_store<1>(v, partial, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ clover observables
// Per site and plane (i < j): the clover C_ij = P_ij + P_{j,-i} + P_{-i,-j} + P_{-j,i}
// (LinkMatrix::clover, src/field.rs:806-820; pij with U_{-mu}(x) = U_mu(x - mu)^dag), the field
// strength F_ij = (C_ij - C_ji) / (8 size^2) = (C_ij - C_ij^dag) / (8 size^2) (f_mu_nu, :822-835; the
// leaves of C_ji are the reversed leaves of C_ij) and the magnetic field
// B_k = (1/2i) sum_{i,j} eps(k,i,j) F_ij = -i sum_{i<j} eps(k,i,j) F_ij (magnetic_field, :849-871,
// with eps the three-index levi_civita of src/utils.rs:306-318).  Hi parts; double output in the
// serde 3x3 layout: f_out[site][plane][18], b_out[site][k][18].
template <int D, typename T>
__global__ void __launch_bounds__(128) k_clover_fields(const V2<T> *__restrict__ U, Geo<D> g, double *f_out,
                                                       double *b_out, double inv_8s2) {
    constexpr int NP = D * (D - 1) / 2;
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    if (site >= g.V) return;
    uint32_t c[D];
    site_coords(g, site, c);
    auto ld = [&](uint32_t x, int dir, mat3<T> &m) { load_link<T>(U, tix(x, D * 9, dir * 9), m); };
    auto store18 = [](double *dst, const mat3<double> &m) {
#pragma unroll
        for (int col = 0; col < 3; ++col)
#pragma unroll
            for (int row = 0; row < 3; ++row) {
                dst[(col * 3 + row) * 2] = m.e[row * 3 + col].re;
                dst[(col * 3 + row) * 2 + 1] = m.e[row * 3 + col].im;
            }
    };
    // B accumulates in its output rows (each thread owns its site's rows)
    if (b_out)
        for (int q = 0; q < D * 18; ++q) b_out[(size_t)site * D * 18 + q] = 0.0;
    int p = 0;
#pragma unroll 1
    for (int i = 0; i < D; ++i) {
#pragma unroll 1
        for (int j = i + 1; j < D; ++j, ++p) {
            const uint32_t xpi = fwd(g, site, c[i], i), xmi = bwd(g, site, c[i], i);
            const uint32_t xpj = fwd(g, site, c[j], j), xmj = bwd(g, site, c[j], j);
            const uint32_t xpj_mi = bwd(g, xpj, c[i], i), xmi_mj = bwd(g, xmi, c[j], j);
            const uint32_t xpi_mj = bwd(g, xpi, c[j], j);
            mat3<T> a, bb, t1, t2, leaf, cl;
            // P_ij = U_i(x) U_j(x+i) U_i(x+j)^dag U_j(x)^dag
            ld(site, i, a);
            ld(xpi, j, bb);
            mul_nn(a, bb, t1);
            ld(xpj, i, a);
            mul_na(t1, a, t2);
            ld(site, j, a);
            mul_na(t2, a, cl);
            // P_{j,-i} = U_j(x) U_i(x+j-i)^dag U_j(x-i)^dag U_i(x-i)
            ld(site, j, a);
            ld(xpj_mi, i, bb);
            mul_na(a, bb, t1);
            ld(xmi, j, a);
            mul_na(t1, a, t2);
            ld(xmi, i, a);
            mul_nn(t2, a, leaf);
#pragma unroll
            for (int k = 0; k < 9; ++k) cl.e[k] = cmk(cl.e[k].re + leaf.e[k].re, cl.e[k].im + leaf.e[k].im);
            // P_{-i,-j} = U_i(x-i)^dag U_j(x-i-j)^dag U_i(x-i-j) U_j(x-j)
            ld(xmi_mj, j, a);
            ld(xmi, i, bb);
            mul_nn(a, bb, t1); // (U_i(x-i)^dag U_j(x-i-j)^dag)^dag
            ld(xmi_mj, i, a);
            mul_an(t1, a, t2);
            ld(xmj, j, a);
            mul_nn(t2, a, leaf);
#pragma unroll
            for (int k = 0; k < 9; ++k) cl.e[k] = cmk(cl.e[k].re + leaf.e[k].re, cl.e[k].im + leaf.e[k].im);
            // P_{-j,i} = U_j(x-j)^dag U_i(x-j) U_j(x+i-j) U_i(x)^dag
            ld(xmj, j, a);
            ld(xmj, i, bb);
            mul_an(a, bb, t1);
            ld(xpi_mj, j, a);
            mul_nn(t1, a, t2);
            ld(site, i, a);
            mul_na(t2, a, leaf);
#pragma unroll
            for (int k = 0; k < 9; ++k) cl.e[k] = cmk(cl.e[k].re + leaf.e[k].re, cl.e[k].im + leaf.e[k].im);
            // F_ij = (C - C^dag) / (8 size^2), in double
            mat3<double> f;
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const cpx<T> x = cl.e[r * 3 + q], y = cl.e[q * 3 + r];
                    f.e[r * 3 + q] = cmk(((double)x.re - (double)y.re) * inv_8s2, ((double)x.im + (double)y.im) * inv_8s2);
                }
            if (f_out) store18(f_out + ((size_t)site * NP + p) * 18, f);
            // B_k += -i eps(k, i, j) F_ij: -i (a + ib) = b - ia
            if (b_out)
                for (int k = 0; k < D; ++k) {
                    if (k == i || k == j) continue;
                    const double eps = (double)(((i > k) - (i < k)) * ((j > k) - (j < k)) * ((j > i) - (j < i)));
                    double *dst = b_out + ((size_t)site * D + k) * 18;
#pragma unroll
                    for (int col = 0; col < 3; ++col)
#pragma unroll
                        for (int row = 0; row < 3; ++row) {
                            const cpx<double> x = f.e[row * 3 + col];
                            dst[(col * 3 + row) * 2] += eps * x.im;
                            dst[(col * 3 + row) * 2 + 1] -= eps * x.re;
                        }
                }
        }
    }
}

// sum of squares of an E-field (hi + lo), hamiltonian_efield before the beta/2 factor
template <typename T, bool COMP>
__global__ void __launch_bounds__(256) k_sum_squares(const T *__restrict__ x, size_t n, double *__restrict__ partial) {
    T acc = T(0);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const T y = x[i];
        if (COMP) acc = fma(y, y, fma(T(2) * y, x[n + i], acc));
        else acc = fma(y, y, acc);
    }
    double v[1] = {(double)acc};
    block_reduce_store<1>(v, partial, blockIdx.x, gridDim.x);
}

// sum over E-field components of (e' - e)(e' + e), i.e. Delta of the sum of squares, with
// e' - e including the compensated parts (Delta hamiltonian_efield = beta/2 times it)
template <typename T, bool COMP>
__global__ void __launch_bounds__(256) k_sum_squares_delta(const T *__restrict__ eo, const T *__restrict__ en, size_t n,
                                                           double *__restrict__ partial) {
    // row 0: sum (e' - e)(e' + e); row 1: sum e^2 of eo, element for element and in the order
    // of k_sum_squares on the same launch shape, so it equals k_sum_squares(eo) bitwise
    T acc = T(0), sq = T(0);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const T a = eo[i], b = en[i];
        T d = b - a;
        if (COMP) {
            const T al = eo[n + i];
            d += en[n + i] - al;
            sq = fma(a, a, fma(T(2) * a, al, sq));
        } else {
            sq = fma(a, a, sq);
        }
        acc = fma(d, a + b, acc);
    }
    double v[2] = {(double)acc, (double)sq};
    block_reduce_store<2>(v, partial, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ reprojection
// orthonormalize_matrix (src/su3.rs:290-309), computed in double for every storage type:
// v1 = col0 / |col0|, v2 = col1 - v1 (v1^* . col1), normalised, col2 = conj(v1) x conj(v2);
// a vector whose norm is <= f64::EPSILON is kept unnormalised (try_normalize).
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_normalize(V2<T> *__restrict__ U, Geo<D> g, size_t ulo) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    const int mu = blockIdx.y;
    if (site >= g.V) return;
    const size_t p0 = tix(site, D * 9, mu * 9);
    double r1[3], i1[3], r2[3], i2[3];
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        const V2<T> a = U[p0 + link_off<T>(p0, (row * 3 + 0))];
        const V2<T> b = U[p0 + link_off<T>(p0, (row * 3 + 1))];
        r1[row] = a.x;
        i1[row] = a.y;
        r2[row] = b.x;
        i2[row] = b.y;
        if (COMP) {
            const V2<T> al = U[ulo + p0 + link_off<T>(p0, (row * 3 + 0))];
            const V2<T> bl = U[ulo + p0 + link_off<T>(p0, (row * 3 + 1))];
            r1[row] += al.x;
            i1[row] += al.y;
            r2[row] += bl.x;
            i2[row] += bl.y;
        }
    }
    const double eps = 2.220446049250313e-16;
    double n1 = sqrt(r1[0] * r1[0] + i1[0] * i1[0] + r1[1] * r1[1] + i1[1] * i1[1] + r1[2] * r1[2] + i1[2] * i1[2]);
    if (n1 > eps) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            r1[k] /= n1;
            i1[k] /= n1;
        }
    }
    // proj = sum_k conj(v1_k) v2_k
    double pr = 0.0, pi = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        pr += r1[k] * r2[k] + i1[k] * i2[k];
        pi += r1[k] * i2[k] - i1[k] * r2[k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double tr = r1[k] * pr - i1[k] * pi;
        const double ti = r1[k] * pi + i1[k] * pr;
        r2[k] -= tr;
        i2[k] -= ti;
    }
    const double n2 =
        sqrt(r2[0] * r2[0] + i2[0] * i2[0] + r2[1] * r2[1] + i2[1] * i2[1] + r2[2] * r2[2] + i2[2] * i2[2]);
    if (n2 > eps) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            r2[k] /= n2;
            i2[k] /= n2;
        }
    }
    // col2 = conj(v1) x conj(v2): (a x b)_k with a = conj(v1), b = conj(v2)
    double r3[3], i3[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
        const double xr = r1[k1] * r2[k2] - i1[k1] * i2[k2];
        const double xi = -(r1[k1] * i2[k2] + i1[k1] * r2[k2]);
        const double yr = r1[k2] * r2[k1] - i1[k2] * i2[k1];
        const double yi = -(r1[k2] * i2[k1] + i1[k2] * r2[k1]);
        r3[k] = xr - yr;
        i3[k] = xi - yi;
    }
    const double *cols_r[3] = {r1, r2, r3};
    const double *cols_i[3] = {i1, i2, i3};
#pragma unroll
    for (int row = 0; row < 3; ++row)
#pragma unroll
        for (int col = 0; col < 3; ++col) {
            V2<T> h, l;
            split(cols_r[col][row], h.x, l.x);
            split(cols_i[col][row], h.y, l.y);
            U[p0 + link_off<T>(p0, (row * 3 + col))] = h;
            if (COMP) U[ulo + p0 + link_off<T>(p0, (row * 3 + col))] = l;
        }
}

// ------------------------------------------------------------------ layout conversion
// host serde layout (double AoS, column-major complex 3x3 per link) <-> device SoA planes
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_links_from_aos(const double *__restrict__ aos, V2<T> *__restrict__ U,
                                                        uint32_t V, size_t ulo) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    const int mu = blockIdx.y;
    if (site >= V) return;
    const double *src = aos + ((size_t)site * D + mu) * 18;
    const size_t p0 = tix(site, D * 9, mu * 9);
#pragma unroll
    for (int col = 0; col < 3; ++col)
#pragma unroll
        for (int row = 0; row < 3; ++row) {
            V2<T> h, l;
            split(src[(col * 3 + row) * 2], h.x, l.x);
            split(src[(col * 3 + row) * 2 + 1], h.y, l.y);
            const size_t idx = p0 + link_off<T>(p0, (row * 3 + col));
            U[idx] = h;
            if (COMP) U[ulo + idx] = l;
        }
}
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_links_to_aos(const V2<T> *__restrict__ U, double *__restrict__ aos,
                                                      uint32_t V, size_t ulo) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    const int mu = blockIdx.y;
    if (site >= V) return;
    double *dst = aos + ((size_t)site * D + mu) * 18;
    const size_t p0 = tix(site, D * 9, mu * 9);
#pragma unroll
    for (int col = 0; col < 3; ++col)
#pragma unroll
        for (int row = 0; row < 3; ++row) {
            const size_t idx = p0 + link_off<T>(p0, (row * 3 + col));
            const V2<T> v = U[idx];
            double re = (double)v.x, im = (double)v.y;
            if (COMP) {
                const V2<T> l = U[ulo + idx];
                re += (double)l.x;
                im += (double)l.y;
            }
            dst[(col * 3 + row) * 2] = re;
            dst[(col * 3 + row) * 2 + 1] = im;
        }
}
// LO = false (compensated storage only): hi = fl(x) and lo = 0, for a field that the Gauss projection
// takes next -- its sweeps read the hi parts only and clear the lo parts when they finish -- so the
// three FP64 operations per value of the exact lo are not spent.
template <int D, typename T, bool COMP, bool LO = true>
__global__ void __launch_bounds__(128) k_efield_from_aos(const double *__restrict__ aos, T *__restrict__ E,
                                                         uint32_t V, size_t elo) {
    // one thread per link, the D directions of a site on consecutive threads: a warp reads 2 KB of the
    // reference layout contiguously (128-bit loads)
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t site = t / D;
    const int mu = (int)(t % D);
    if (site >= V) return;
    const double2 *src = reinterpret_cast<const double2 *>(aos + (size_t)t * 8);
    T h[8], l[8];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const double2 v = __ldg(src + j);
        if (LO) {
            split(v.x, h[2 * j], l[2 * j]);
            split(v.y, h[2 * j + 1], l[2 * j + 1]);
        } else {
            h[2 * j] = (T)v.x;
            h[2 * j + 1] = (T)v.y;
            l[2 * j] = T(0);
            l[2 * j + 1] = T(0);
        }
    }
    const size_t ei = tix(site, D * 8, mu * 8);
    store_efield<T>(E, ei, h);
    if (COMP) store_efield<T>(E + elo, ei, l);
}
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_efield_to_aos(const T *__restrict__ E, double *__restrict__ aos,
                                                       uint32_t V, size_t elo) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t site = t / D;
    const int mu = (int)(t % D);
    if (site >= V) return;
    const size_t ei = tix(site, D * 8, mu * 8);
    T h[8], l[8];
    load_efield<T>(E, ei, h);
    if (COMP) load_efield<T>(E + elo, ei, l);
    double2 *dst = reinterpret_cast<double2 *>(aos + (size_t)t * 8);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        double x0 = (double)h[2 * j], x1 = (double)h[2 * j + 1];
        if (COMP) {
            x0 += (double)l[2 * j];
            x1 += (double)l[2 * j + 1];
        }
        dst[j] = make_double2(x0, x1);
    }
}
// G(x) as its 8 su(3) coefficients g^a = 2 Re Tr(T^a G(x))
template <typename T>
__global__ void __launch_bounds__(256) k_gauss_to_aos(const T *__restrict__ G, double *__restrict__ out, uint32_t V) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    if (site >= V) return;
    mat3<T> m;
    herm_load(G, site, m);
    T gc[8];
    two_re_tr_generators(m, gc);
#pragma unroll
    for (int a = 0; a < 8; ++a) out[(size_t)site * 8 + a] = (double)gc[a];
}

// identity links (hi array; the lo array, when present, is cleared by the caller)
template <int D, typename T>
__global__ void __launch_bounds__(128) k_links_identity(V2<T> *__restrict__ U, uint32_t V) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    const int mu = blockIdx.y;
    if (site >= V) return;
    const size_t p0 = tix(site, D * 9, mu * 9);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        V2<T> v;
        v.x = (k == 0 || k == 4 || k == 8) ? T(1) : T(0);
        v.y = T(0);
        U[p0 + link_off<T>(p0, k)] = v;
    }
}

// ------------------------------------------------------------------ Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror & Shaw (SC'11): 10 rounds of the
// 4x32 S-box with multipliers 0xD2511F53 / 0xCD9E8D57 and Weyl key increments
// 0x9E3779B9 / 0xBB67AE85.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}
// [0,1) with 53 random bits
__device__ __forceinline__ double u01_53(uint32_t hi, uint32_t lo) {
    const uint64_t v = (((uint64_t)hi << 32) | lo) >> 11;
    return (double)v * 0x1.0p-53;
}
// [0,1) with 24 random bits
__device__ __forceinline__ float u01_24(uint32_t x) { return (float)(x >> 8) * 0x1.0p-24f; }

// Box-Muller pair from two uniforms in [0,1)
__device__ __forceinline__ void box_muller(double u1, double u2, double &z0, double &z1) {
    const double r = sqrt(-2.0 * log(1.0 - u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    z0 = r * c;
    z1 = r * s;
}
__device__ __forceinline__ void box_muller(float u1, float u2, float &z0, float &z1) {
    const float r = sqrtf(-2.0f * logf(1.0f - u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

// E^a(x, mu) ~ Normal(0, sd), independent per (link, a); counter = (link, ctr_lo, ctr_hi, call).
// FP64 states draw 53-bit uniforms and double-precision Box-Muller; FP32 states 24-bit ones.
template <int D, typename T, bool COMP>
__device__ __forceinline__ void efield_normal_link(T *__restrict__ E, uint32_t site, int mu, uint2 key,
                                                   uint32_t ctr_lo, uint32_t ctr_hi, T sd, size_t elo) {
    const uint32_t link = site * D + mu;
    T z[8];
    if (sizeof(T) == 8) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint4 r = philox4x32_10(make_uint4(link, ctr_lo, ctr_hi, (uint32_t)j), key);
            double a, b;
            box_muller(u01_53(r.x, r.y), u01_53(r.z, r.w), a, b);
            z[2 * j] = (T)a;
            z[2 * j + 1] = (T)b;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const uint4 r = philox4x32_10(make_uint4(link, ctr_lo, ctr_hi, (uint32_t)j), key);
            float a, b, c2, d2;
            box_muller(u01_24(r.x), u01_24(r.y), a, b);
            box_muller(u01_24(r.z), u01_24(r.w), c2, d2);
            z[4 * j] = (T)a;
            z[4 * j + 1] = (T)b;
            z[4 * j + 2] = (T)c2;
            z[4 * j + 3] = (T)d2;
        }
    }
    const size_t ei = tix(site, D * 8, mu * 8);
    T h[8], l[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        h[a] = z[a] * sd;
        l[a] = T(0);
    }
    store_efield<T>(E, ei, h);
    if (COMP) store_efield<T>(E + elo, ei, l);
}
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_efield_normal(T *__restrict__ E, uint32_t V, uint2 key, uint32_t ctr_lo,
                                                       uint32_t ctr_hi, T sd) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    const int mu = blockIdx.y;
    if (site >= V) return;
    efield_normal_link<D, T, COMP>(E, site, mu, key, ctr_lo, ctr_hi, sd, (size_t)tiles_of(V) * D * 8 * kTile);
}

// random_su3 (src/su3.rs:322-355) per link: two complex 3-vectors with Uniform(-1,1)
// entries, redrawn while |v1| <= eps or |v1 . v2| <= eps; written as columns 0 and 1, which
// k_normalize then turns into Gram-Schmidt vectors and col2 = conj(v1) x conj(v2).
template <int D, typename T, bool COMP>
__global__ void __launch_bounds__(128) k_links_random(V2<T> *__restrict__ U, uint32_t V, uint2 key, size_t ulo) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    const int mu = blockIdx.y;
    if (site >= V) return;
    const uint32_t link = site * D + mu;
    const double eps = 2.220446049250313e-16;
    double r1[3], i1[3], r2[3], i2[3];
    uint32_t call = 0;
    auto draw6 = [&](double *re, double *im) {
        // 6 uniforms from 3 Philox blocks (53 bits each)
        double u[6];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const uint4 r = philox4x32_10(make_uint4(link, call++, 0x53553300u, 0u), key);
            u[2 * j] = u01_53(r.x, r.y);
            u[2 * j + 1] = u01_53(r.z, r.w);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            re[k] = u[2 * k] * 2.0 - 1.0;
            im[k] = u[2 * k + 1] * 2.0 - 1.0;
        }
    };
    for (int tries = 0; tries < 64; ++tries) {
        draw6(r1, i1);
        const double n = r1[0] * r1[0] + i1[0] * i1[0] + r1[1] * r1[1] + i1[1] * i1[1] + r1[2] * r1[2] + i1[2] * i1[2];
        if (sqrt(n) > eps) break;
    }
    for (int tries = 0; tries < 64; ++tries) {
        draw6(r2, i2);
        double dr = 0.0, di = 0.0; // non-conjugating dot
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            dr += r1[k] * r2[k] - i1[k] * i2[k];
            di += r1[k] * i2[k] + i1[k] * r2[k];
        }
        if (hypot(dr, di) > eps) break;
    }
    const size_t p0 = tix(site, D * 9, mu * 9);
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        V2<T> a, b, al, bl;
        split(r1[row], a.x, al.x);
        split(i1[row], a.y, al.y);
        split(r2[row], b.x, bl.x);
        split(i2[row], b.y, bl.y);
        U[p0 + link_off<T>(p0, (row * 3 + 0))] = a;
        U[p0 + link_off<T>(p0, (row * 3 + 1))] = b;
        if (COMP) {
            U[ulo + p0 + link_off<T>(p0, (row * 3 + 0))] = al;
            U[ulo + p0 + link_off<T>(p0, (row * 3 + 1))] = bl;
        }
    }
}

} // namespace lq
