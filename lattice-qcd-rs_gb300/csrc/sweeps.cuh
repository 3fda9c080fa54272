// sweeps.cuh -- the reference's local Monte Carlo methods on the device: MetropolisHastingsSweep
// and HeatBathSweep (src/simulation/monte_carlo/metropolis_hastings_sweep.rs, heat_bath.rs).
//
// The reference updates the links one after another in lattice order.  Here a sweep runs in
// checkerboard order: for each direction mu, every link (x, mu) with sum_i x_i even, then every one
// with it odd.  The staple of (x, mu) contains U_mu(x +- nu) (the other class) and links of other
// directions only, so a class updates at once; L must be even for the classes to alternate across
// the periodic boundary.  Per link the update is the reference's, in double for every storage form
// (the stored value is split back into hi + lo), with random numbers from a Philox4x32-10 stream per
// link: counter blocks (link, sweep lo, sweep hi, 0x80000000 + call), two 53-bit uniforms per block.
// Every rejection loop is bounded (kMaxRedraws draws; the reference loops without a bound).
#pragma once
#include "kernels.cuh"

namespace lq {

constexpr int kMaxRedraws = 10000;

// f64::is_normal: finite, not zero, not subnormal (NaN fails both comparisons)
__device__ __forceinline__ bool is_normal_d(double x) {
    const double a = fabs(x);
    return a >= 2.2250738585072014e-308 && a <= 1.7976931348623157e308;
}

struct LinkRng {
    uint2 key;
    uint32_t link, s_lo, s_hi, call;
    double buf;
    bool has;
    __device__ double next() {
        if (has) {
            has = false;
            return buf;
        }
        const uint4 r = philox4x32_10(make_uint4(link, s_lo, s_hi, 0x80000000u + call++), key);
        buf = u01_53(r.z, r.w);
        has = true;
        return u01_53(r.x, r.y);
    }
    // Uniform::new(a, b): a + (b - a) u, without contraction
    __device__ double uniform(double a, double b) { return __dadd_rn(a, __dmul_rn(b - a, next())); }
    __device__ double open_closed01() { return 1.0 - next(); }
    __device__ bool half() { return next() < 0.5; }
};

struct m2d {
    cpx<double> e[4]; // row-major 2x2
};
__device__ __forceinline__ cpx<double> cmul(cpx<double> a, cpx<double> b) {
    return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ cpx<double> cadd(cpx<double> a, cpx<double> b) { return cmk(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ m2d mul2(const m2d &a, const m2d &b) {
    m2d r;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) r.e[i * 2 + j] = cadd(cmul(a.e[i * 2], b.e[j]), cmul(a.e[i * 2 + 1], b.e[2 + j]));
    return r;
}

// su2::complex_matrix_from_vec (src/su2.rs:134-140): x0 1 + sum_i PAULI_MATRICES[i] (i x_i), with the
// reference's constants, in which PAULI_3 is the identity (src/su2.rs:13-49):
//   [[x0 + i x3, x2 + i x1], [-x2 + i x1, x0 + i x3]]
__device__ __forceinline__ m2d complex_matrix_from_vec(double x0, const double *x) {
    m2d r;
    r.e[0] = cmk(x0, x[2]);
    r.e[1] = cmk(x[1], x[0]);
    r.e[2] = cmk(-x[1], x[0]);
    r.e[3] = cmk(x0, x[2]);
    return r;
}
// su2::random_su2_close_to_unity (src/su2.rs:80-100)
__device__ __forceinline__ m2d random_su2_close_to_unity(double spread, LinkRng &rng) {
    double r[3], x[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = rng.uniform(-1.0, 1.0);
    const double n = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) x[i] = (n > 2.220446049250313e-16 ? r[i] / n : r[i]) * spread;
    const double x0u = sqrt(1.0 - (x[0] * x[0] + x[1] * x[1] + x[2] * x[2]));
    const double x0 = rng.half() ? x0u : -x0u;
    return complex_matrix_from_vec(x0, x);
}
// su2::random_su2 (src/su2.rs:200-216)
__device__ __forceinline__ m2d random_su2(LinkRng &rng) {
    cpx<double> v[2];
    double n = 0.0;
    for (int tries = 0; tries < kMaxRedraws; ++tries) {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const double re = rng.uniform(-1.0, 1.0);
            v[k] = cmk(re, rng.uniform(-1.0, 1.0));
        }
        n = sqrt(v[0].re * v[0].re + v[0].im * v[0].im + (v[1].re * v[1].re + v[1].im * v[1].im));
        if (is_normal_d(n)) break;
    }
    const cpx<double> a = cmk(v[0].re / n, v[0].im / n), b = cmk(v[1].re / n, v[1].im / n);
    m2d r;
    r.e[0] = a;
    r.e[1] = b;
    r.e[2] = cmk(-b.re, b.im);
    r.e[3] = cmk(a.re, -a.im);
    return r;
}
// SU(2) block embedded at rows / columns (p, q) of the identity (su3::get_r, get_s, get_t)
__device__ __forceinline__ void embed(const m2d &m, int p, int q, mat3<double> &r) {
    mat_identity(r);
    r.e[p * 3 + p] = m.e[0];
    r.e[p * 3 + q] = m.e[1];
    r.e[q * 3 + p] = m.e[2];
    r.e[q * 3 + q] = m.e[3];
}
// su2::project_to_su2_unorm of the (p, q) sub-block: b - b^dag + 1 conj(Tr b)
__device__ __forceinline__ m2d su2_unorm(const mat3<double> &in, int p, int q) {
    m2d b;
    b.e[0] = in.e[p * 3 + p];
    b.e[1] = in.e[p * 3 + q];
    b.e[2] = in.e[q * 3 + p];
    b.e[3] = in.e[q * 3 + q];
    const cpx<double> tr = cmk(b.e[0].re + b.e[3].re, -(b.e[0].im + b.e[3].im));
    m2d r;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const cpx<double> x = b.e[i * 2 + j], y = b.e[j * 2 + i];
            cpx<double> d = cmk(x.re - y.re, x.im + y.im);
            if (i == j) d = cadd(d, tr);
            r.e[i * 2 + j] = d;
        }
    return r;
}
// su3::random_su3_close_to_unity (src/su3.rs:385-398)
__device__ __forceinline__ void random_su3_close_to_unity(double spread, LinkRng &rng, mat3<double> &x) {
    mat3<double> r, s, t, rs;
    embed(random_su2_close_to_unity(spread, rng), 0, 1, r);
    embed(random_su2_close_to_unity(spread, rng), 0, 2, s);
    embed(random_su2_close_to_unity(spread, rng), 1, 2, t);
    mul_nn(r, s, rs);
    mul_nn(rs, t, x);
    if (rng.half()) {
        mat3<double> a = x;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) x.e[i * 3 + j] = cmk(a.e[j * 3 + i].re, -a.e[j * 3 + i].im);
    }
}
// statistics::ModifiedNormal, HeatBathDistributionNorm, HeatBathDistribution
// (src/statistics/distribution.rs:76-101, :320-350, :199-218)
__device__ __forceinline__ double modified_normal(double param, LinkRng &rng) {
    double r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = rng.open_closed01();
    const double c = cos(2.0 * 3.141592653589793 * r[1]);
    return sqrt(-(log(r[0]) + c * c * log(r[2])) / (2.0 * param));
}
__device__ __forceinline__ m2d heat_bath_sample(double param, LinkRng &rng) {
    double x0 = 1.0;
    for (int tries = 0; tries < kMaxRedraws; ++tries) {
        const double r = rng.uniform(0.0, 1.0);
        const double lambda = modified_normal(param, rng);
        if (r * r <= 1.0 - lambda * lambda) {
            x0 = 1.0 - 2.0 * lambda * lambda;
            break;
        }
    }
    double x[3], n = 0.0;
    for (int tries = 0; tries < kMaxRedraws; ++tries) {
#pragma unroll
        for (int i = 0; i < 3; ++i) x[i] = rng.uniform(-1.0, 1.0);
        n = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        if (n > 2.220446049250313e-16) break;
    }
    const double f = sqrt(1.0 - x0 * x0);
#pragma unroll
    for (int i = 0; i < 3; ++i) x[i] = x[i] / n * f;
    return complex_matrix_from_vec(x0, x);
}
// HeatBathSweep::heat_bath_su2 (heat_bath.rs:71-86)
__device__ __forceinline__ m2d heat_bath_su2(const m2d &st, double beta, LinkRng &rng) {
    const cpx<double> det = cmk(st.e[0].re * st.e[3].re - st.e[0].im * st.e[3].im -
                                    (st.e[2].re * st.e[1].re - st.e[2].im * st.e[1].im),
                                0.0);
    const double k = sqrt(det.re);
    if (is_normal_d(k)) {
        m2d v;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const cpx<double> z = st.e[j * 2 + i]; // adjoint
                v.e[i * 2 + j] = cmk(z.re * k / (k * k), -z.im * k / (k * k));
            }
        return mul2(heat_bath_sample(beta * k, rng), v);
    }
    return random_su2(rng);
}

// the link (site, mu) and its neighbours as double (hi + lo with compensated storage)
template <typename T, bool COMP>
__device__ __forceinline__ void load_link_d(const V2<T> *__restrict__ U, size_t ulo, size_t i, mat3<double> &m) {
    mat3<T> h, l;
    load_link<T>(U, i, h);
    if (COMP) load_link<T>(U + ulo, i, l);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        double re = (double)h.e[k].re, im = (double)h.e[k].im;
        if (COMP) {
            re += (double)l.e[k].re;
            im += (double)l.e[k].im;
        }
        m.e[k] = cmk(re, im);
    }
}
template <typename T, bool COMP>
__device__ __forceinline__ void store_link_d(V2<T> *__restrict__ U, size_t ulo, size_t i, const mat3<double> &m) {
    mat3<T> h, l;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        split(m.e[k].re, h.e[k].re, l.e[k].re);
        split(m.e[k].im, h.e[k].im, l.e[k].im);
    }
    store_link<T>(U, i, h);
    if (COMP) store_link<T>(U + ulo, i, l);
}
// the staple of the Monte Carlo methods (src/simulation/monte_carlo/mod.rs:339-362):
// sum over nu != mu of S_mu,nu(x)^dag + U_nu(x+mu-nu)^dag U_mu(x-nu)^dag U_nu(x-nu)
template <int D, typename T, bool COMP>
__device__ __forceinline__ void mc_staple(const V2<T> *__restrict__ U, size_t ulo, const Geo<D> &g, uint32_t site,
                                          const uint32_t *c, int mu, mat3<double> &sum) {
    const uint32_t xpmu = fwd(g, site, c[mu], mu);
    mat_zero(sum);
#pragma unroll 1
    for (int nu = 0; nu < D; ++nu) {
        if (nu == mu) continue;
        mat3<double> a, b, t, term;
        // S^dag = U_nu(x+mu) U_mu(x+nu)^dag U_nu(x)^dag
        load_link_d<T, COMP>(U, ulo, tix(xpmu, D * 9, nu * 9), a);
        load_link_d<T, COMP>(U, ulo, tix(fwd(g, site, c[nu], nu), D * 9, mu * 9), b);
        mul_na(a, b, t);
        load_link_d<T, COMP>(U, ulo, tix(site, D * 9, nu * 9), a);
        mul_na(t, a, term);
        // U_nu(x+mu-nu)^dag U_mu(x-nu)^dag U_nu(x-nu) = (U_mu(x-nu) U_nu(x+mu-nu))^dag U_nu(x-nu)
        const uint32_t xmnu = bwd(g, site, c[nu], nu);
        load_link_d<T, COMP>(U, ulo, tix(bwd(g, xpmu, c[nu], nu), D * 9, nu * 9), a);
        load_link_d<T, COMP>(U, ulo, tix(xmnu, D * 9, mu * 9), b);
        mat3<double> ba;
        mul_nn(b, a, ba);
        load_link_d<T, COMP>(U, ulo, tix(xmnu, D * 9, nu * 9), a);
        mul_an(ba, a, t);
#pragma unroll
        for (int k = 0; k < 9; ++k)
            sum.e[k] = cmk(sum.e[k].re + (term.e[k].re + t.e[k].re), sum.e[k].im + (term.e[k].im + t.e[k].im));
    }
}

enum : int { MC_METROPOLIS = 0, MC_HEAT_BATH = 1, MC_OVERRELAX_ROTATION = 2, MC_OVERRELAX_REVERSE = 3 };

// ---- overrelaxation (src/simulation/monte_carlo/overrelaxation.rs), in double ----
// Both methods use the singular value decomposition a = U S V^dag of a = staple^dag (nalgebra's SVD
// in the reference), taken here from the eigen-decomposition of the Hermitian a^dag a = V S^2 V^dag
// by cyclic complex Jacobi rotations (Golub & Van Loan, Matrix Computations, section 8.5: the phase
// of the off-diagonal element removed first, then the real rotation with
// tan 2 theta = 2 |h_pq| / (h_qq - h_pp)), kJacobiSweeps = 5 sweeps over the pairs (0,1), (0,2),
// (1,2), and U = a V S^-1 (cyclic Jacobi converges quadratically: on random staples and on staples
// with singular values 1e-9 apart, 4 sweeps already give the updates of 8 to 2e-15).  For distinct singular values both updates are independent of the SVD's phase and
// ordering freedom, so they are the reference's:
//   rotation (:92-104): rot = U V^dag, U' = rot U^dag rot
//   reverse  (:160-172): U' = U reverse(U^dag L V) V^dag, reverse negating the off-diagonal entries
//                        (su3.rs:705-714)
// The update divides by the smallest singular value of the staple and so magnifies rounding
// differences; everything here, the staple included, is evaluated in the operation order of the
// oracle's restatement with separately rounded products and sums (no fused multiply-add), which keeps
// the FP64 form equal to it.
struct XD {
    // complex arithmetic as the textbook product and sum, each operation rounded
    static __device__ __forceinline__ cpx<double> mul(cpx<double> a, cpx<double> b) {
        return cmk(__dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im)),
                   __dadd_rn(__dmul_rn(a.re, b.im), __dmul_rn(a.im, b.re)));
    }
    static __device__ __forceinline__ cpx<double> add(cpx<double> a, cpx<double> b) {
        return cmk(__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im));
    }
    // r = a b, each entry summed over k = 0, 1, 2 in that order
    static __device__ void mm(const mat3<double> &a, const mat3<double> &b, mat3<double> &r) {
        mat3<double> t;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                cpx<double> x = mul(a.e[i * 3], b.e[j]);
                x = add(x, mul(a.e[i * 3 + 1], b.e[3 + j]));
                x = add(x, mul(a.e[i * 3 + 2], b.e[6 + j]));
                t.e[i * 3 + j] = x;
            }
        r = t;
    }
    static __device__ __forceinline__ void adj(const mat3<double> &a, mat3<double> &r) {
        mat3<double> t;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) t.e[i * 3 + j] = cmk(a.e[j * 3 + i].re, -a.e[j * 3 + i].im);
        r = t;
    }
    static __device__ __forceinline__ void madd(const mat3<double> &a, const mat3<double> &b, mat3<double> &r) {
#pragma unroll
        for (int k = 0; k < 9; ++k) r.e[k] = add(a.e[k], b.e[k]);
    }
};

// the Monte Carlo staple of mc_staple, in the oracle's order: for nu != mu ascending,
//   sum += ((U_nu(x) U_mu(x+nu)) U_nu(x+mu)^dag)^dag + (U_nu(x+mu-nu)^dag U_mu(x-nu)^dag) U_nu(x-nu)
template <int D, typename T, bool COMP>
__device__ void mc_staple_exact(const V2<T> *__restrict__ U, size_t ulo, const Geo<D> &g, uint32_t site,
                                const uint32_t *c, int mu, mat3<double> &sum) {
    const uint32_t xpmu = fwd(g, site, c[mu], mu);
    mat_zero(sum);
#pragma unroll 1
    for (int nu = 0; nu < D; ++nu) {
        if (nu == mu) continue;
        mat3<double> a, b, t, el1, u1, u2, term;
        load_link_d<T, COMP>(U, ulo, tix(site, D * 9, nu * 9), a);
        load_link_d<T, COMP>(U, ulo, tix(fwd(g, site, c[nu], nu), D * 9, mu * 9), b);
        XD::mm(a, b, t);
        load_link_d<T, COMP>(U, ulo, tix(xpmu, D * 9, nu * 9), a);
        XD::adj(a, b);
        XD::mm(t, b, a);
        XD::adj(a, el1);
        const uint32_t xmnu = bwd(g, site, c[nu], nu);
        load_link_d<T, COMP>(U, ulo, tix(bwd(g, xpmu, c[nu], nu), D * 9, nu * 9), a);
        XD::adj(a, u1);
        load_link_d<T, COMP>(U, ulo, tix(xmnu, D * 9, mu * 9), a);
        XD::adj(a, u2);
        XD::mm(u1, u2, t);
        load_link_d<T, COMP>(U, ulo, tix(xmnu, D * 9, nu * 9), a);
        XD::mm(t, a, term);
        XD::madd(el1, term, term);
        XD::madd(sum, term, sum);
    }
}

// One Jacobi rotation J in the (P, Q) plane: h <- (J^dag h) J, v <- v J, with J the identity except
// J_PP = cs, J_PQ = sn, J_QP = -sn e^{-i phi}, J_QQ = cs e^{-i phi}.  Only rows P, Q of J^dag h and
// then columns P, Q change; the other entries of the full products are exact products with 1 and sums
// with zeros, so updating just these entries, each in the full product's order, gives the same values.
template <int P, int Q> __device__ __forceinline__ void jacobi_rotate(mat3<double> &h, mat3<double> &v) {
    const cpx<double> hpq = h.e[P * 3 + Q];
    const double c = sqrt(__dadd_rn(__dmul_rn(hpq.re, hpq.re), __dmul_rn(hpq.im, hpq.im)));
    if (!(c > 0.0)) return;
    const cpx<double> phc = cmk(hpq.re / c, -(hpq.im / c)); // e^{-i phi}
    const double tau = __dsub_rn(h.e[Q * 4].re, h.e[P * 4].re) / (2.0 * c);
    const double t = (tau >= 0.0 ? 1.0 : -1.0) / __dadd_rn(fabs(tau), sqrt(__dadd_rn(1.0, __dmul_rn(tau, tau))));
    const double cs = 1.0 / sqrt(__dadd_rn(1.0, __dmul_rn(t, t))), sn = __dmul_rn(t, cs);
    const cpx<double> jpp = cmk(cs, 0.0), jpq = cmk(sn, 0.0);
    const cpx<double> jqp = XD::mul(phc, cmk(-sn, 0.0)), jqq = XD::mul(phc, cmk(cs, 0.0));
    // conjugates: (J^dag)_PP, (J^dag)_PQ = conj(J_QP), (J^dag)_QP = conj(J_PQ), (J^dag)_QQ
    const cpx<double> app = cmk(jpp.re, -jpp.im), apq = cmk(jqp.re, -jqp.im), aqp = cmk(jpq.re, -jpq.im),
                      aqq = cmk(jqq.re, -jqq.im);
#pragma unroll
    for (int k = 0; k < 3; ++k) { // rows P, Q of J^dag h
        const cpx<double> hp = h.e[P * 3 + k], hq = h.e[Q * 3 + k];
        h.e[P * 3 + k] = XD::add(XD::mul(app, hp), XD::mul(apq, hq));
        h.e[Q * 3 + k] = XD::add(XD::mul(aqp, hp), XD::mul(aqq, hq));
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) { // columns P, Q of (J^dag h) J
        const cpx<double> xp = h.e[i * 3 + P], xq = h.e[i * 3 + Q];
        h.e[i * 3 + P] = XD::add(XD::mul(xp, jpp), XD::mul(xq, jqp));
        h.e[i * 3 + Q] = XD::add(XD::mul(xp, jpq), XD::mul(xq, jqq));
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) { // columns P, Q of v J
        const cpx<double> vp = v.e[i * 3 + P], vq = v.e[i * 3 + Q];
        v.e[i * 3 + P] = XD::add(XD::mul(vp, jpp), XD::mul(vq, jqp));
        v.e[i * 3 + Q] = XD::add(XD::mul(vp, jpq), XD::mul(vq, jqq));
    }
}
constexpr int kJacobiSweeps = 5;

__device__ inline void herm3_eigen_jacobi(mat3<double> h, double (&lam)[3], mat3<double> &v) {
    mat_identity(v);
#pragma unroll 1
    for (int sweep = 0; sweep < kJacobiSweeps; ++sweep) {
        jacobi_rotate<0, 1>(h, v);
        jacobi_rotate<0, 2>(h, v);
        jacobi_rotate<1, 2>(h, v);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) lam[k] = h.e[k * 4].re;
}
__device__ inline mat3<double> overrelax_link(const mat3<double> &link, const mat3<double> &staple, int method) {
    mat3<double> a, h, v, u, av, r, x, y;
    XD::adj(staple, a);
    XD::adj(a, x);
    XD::mm(x, a, h); // a^dag a
    double lam[3];
    herm3_eigen_jacobi(h, lam, v);
    XD::mm(a, v, av);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double sv = sqrt(fmax(lam[k], 0.0));
#pragma unroll
        for (int i = 0; i < 3; ++i) u.e[i * 3 + k] = cmk(av.e[i * 3 + k].re / sv, av.e[i * 3 + k].im / sv);
    }
    if (method == MC_OVERRELAX_ROTATION) {
        mat3<double> rot;
        XD::adj(v, x);
        XD::mm(u, x, rot); // U V^dag
        XD::adj(link, x);
        XD::mm(rot, x, y); // rot U^dag
        XD::mm(y, rot, r);
        return r;
    }
    XD::adj(u, x);
    XD::mm(x, link, y); // U^dag L
    XD::mm(y, v, x);    // U^dag L V
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            if (i != j) x.e[i * 3 + j] = cmk(-x.e[i * 3 + j].re, -x.e[i * 3 + j].im);
    XD::mm(u, x, y);
    XD::adj(v, x);
    XD::mm(y, x, r); // U reverse(...) V^dag
    return r;
}

// One checkerboard class of a sweep: links (x, mu) with parity(x) = parity.  Metropolis partials:
// row 0 accepted count, row 1 sum of acceptance probabilities (per block).  The overrelaxation
// updates draw no random numbers.
template <int D, typename T, bool COMP, int ALG>
__global__ void __launch_bounds__(128) k_mc_sweep(V2<T> *__restrict__ U, Geo<D> g, int mu, int parity, double beta,
                                                  uint2 key, uint32_t s_lo, uint32_t s_hi, int n_update,
                                                  double spread, double *__restrict__ partial) {
    // one thread per site of the class: thread t takes row r = 2t / L (the sites with x1.. fixed)
    // and there the j-th site, j = t - r L / 2, whose coordinate sum has the class's parity, so every
    // lane of a warp has a link to update.  Preconditions, checked by the launcher: L even (each row
    // then holds L / 2 sites of either parity) and x0 the fastest coordinate of the site index.
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    uint32_t c[D];
    uint32_t site = 0;
    const bool active = t < (g.V >> 1);
    if (active) {
        const uint32_t row = div_by_L(g, 2u * t);
        site_coords(g, row * g.L, c); // c[0] = 0
        uint32_t q = (uint32_t)parity;
#pragma unroll
        for (int i = 1; i < D; ++i) q += c[i];
        c[0] = 2u * (t - row * (g.L >> 1)) + (q & 1u);
        site = checked_site(row * g.L + c[0], g.V);
    }
    if (active) {
        const size_t ulo = (size_t)tiles_of(g.V) * D * 9 * kTile;
        const size_t ui = tix(site, D * 9, mu * 9);
        LinkRng rng{key, site * D + (uint32_t)mu, s_lo, s_hi, 0u, 0.0, false};
        mat3<double> u, a, out;
        load_link_d<T, COMP>(U, ulo, ui, u);
        if (ALG == MC_METROPOLIS) {
            // MetropolisHastingsSweep::potential_modif and the accept test (metropolis_hastings_sweep.rs:120-172)
            mat3<double> nm = u, r, t;
            for (int k = 0; k < n_update; ++k) {
                random_su3_close_to_unity(spread, rng, r);
                double re[9], im[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    re[q] = r.e[q].re;
                    im[q] = r.e[q].im;
                }
                orthonormalize_d(re, im);
#pragma unroll
                for (int q = 0; q < 9; ++q) r.e[q] = cmk(re[q], im[q]);
                mul_nn(r, nm, t);
                nm = t;
            }
            mc_staple<D, T, COMP>(U, ulo, g, site, c, mu, a);
            // delta_s_old_new_cmp (mod.rs:324-334): -Re Tr((U' - U) A) beta / 3
            mat3<double> d;
#pragma unroll
            for (int q = 0; q < 9; ++q) d.e[q] = cmk(nm.e[q].re - u.e[q].re, nm.e[q].im - u.e[q].im);
            mul_nn(d, a, t);
            const double ds = -(t.e[0].re + t.e[4].re + t.e[8].re) * beta / 3.0;
            const double p = fmax(fmin(exp(-ds), 1.0), 0.0);
            v[1] = p;
            if (p >= 1.0 || rng.next() < p) {
                store_link_d<T, COMP>(U, ulo, ui, nm);
                v[0] = 1.0;
            }
        } else if (ALG == MC_OVERRELAX_ROTATION || ALG == MC_OVERRELAX_REVERSE) {
            // OverrelaxationSweepRotation / OverrelaxationSweepReverse::get_modif (overrelaxation.rs:92-104,
            // :160-172) with the Monte Carlo staple
            mc_staple_exact<D, T, COMP>(U, ulo, g, site, c, mu, a);
            out = overrelax_link(u, a, ALG);
            store_link_d<T, COMP>(U, ulo, ui, out);
        } else {
            // HeatBathSweep::get_modif (heat_bath.rs:88-108): U' = t s r U
            mc_staple<D, T, COMP>(U, ulo, g, site, c, mu, a);
            mat3<double> ua, r, s, t, x, y;
            mul_nn(u, a, ua);
            embed(heat_bath_su2(su2_unorm(ua, 0, 1), beta, rng), 0, 1, r);
            mul_nn(r, u, x);
            mul_nn(x, a, y);
            embed(heat_bath_su2(su2_unorm(y, 0, 2), beta, rng), 0, 2, s);
            mul_nn(s, r, x);
            mul_nn(x, u, y);
            mul_nn(y, a, x);
            embed(heat_bath_su2(su2_unorm(x, 1, 2), beta, rng), 1, 2, t);
            mul_nn(t, s, x);
            mul_nn(x, r, y);
            mul_nn(y, u, out);
            store_link_d<T, COMP>(U, ulo, ui, out);
        }
    }
    if (ALG == MC_METROPOLIS) block_reduce_store<2>(v, partial, blockIdx.x, gridDim.x);
}

} // namespace lq
