/*
 * lq_oracle.cpp -- CPU oracle for the HMC molecular-dynamics path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the CPU baseline
 * of bench.py.  Nothing in the product path links or calls this file.
 *
 * A C++17 restatement of lattice-qcd-rs v0.2.1 (Rust).  Each routine names the
 * reference file:line it follows.  Loop orders, the array-of-structures f64 layout,
 * the per-step allocation of new fields and the operation order inside each
 * formula follow the reference, so that this code is both the parity oracle and a
 * fair stand-in for the reference's CPU cost.  OpenMP parallel loops over sites and
 * links stand in for rayon's `par_iter`/`par_bridge` (src/thread.rs:684-699).
 *
 * Third-party arithmetic restated here (sources not vendored in the reference):
 *  - nalgebra 0.31 3x3 complex products, adjoint, trace, determinant, cross,
 *    try_normalize (src/su3.rs:279-309);
 *  - num-complex textbook complex product;
 *  - rand 0.8 `Uniform<f64>` (53-bit mantissa fill, value0_1 * scale + low) and
 *    `Bernoulli` (p == 1 always true, else u < p);
 *  - Xoshiro256++ / SplitMix64 (Blackman & Vigna) as the seeded generator;
 *  - normals: Box-Muller over the Xoshiro uniforms.  rand_distr's ziggurat is NOT
 *    restated, so random streams are not bit-identical to the Rust crate (parity
 *    of random streams is unpinned); parity tests inject the same buffers into this
 *    oracle and the CUDA library instead.
 *
 * Compiled with -ffp-contract=off so no multiply-add is fused (Rust never fuses),
 * giving identical results on x86-64 and aarch64.
 */
#include "lq_oracle.h"

#include <cmath>
#include <cstring>
#include <vector>
#include <array>
#include <omp.h>

namespace {

constexpr double F64_EPS = 2.220446049250313e-16; /* f64::EPSILON */

struct Cx {
    double re, im;
};
inline Cx cx(double r, double i = 0.0) { return Cx{r, i}; }
inline Cx operator+(Cx a, Cx b) { return Cx{a.re + b.re, a.im + b.im}; }
inline Cx operator-(Cx a, Cx b) { return Cx{a.re - b.re, a.im - b.im}; }
/* num-complex Mul: (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re) */
inline Cx operator*(Cx a, Cx b) { return Cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cx conj(Cx a) { return Cx{a.re, -a.im}; }
inline double modulus(Cx a) { return std::hypot(a.re, a.im); }
inline double modulus_squared(Cx a) { return a.re * a.re + a.im * a.im; }

/* 3x3 complex matrix, m[row][col] */
struct M3 {
    Cx m[3][3];
};

inline M3 zero3() {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = cx(0.0, 0.0);
    return r;
}
inline M3 identity3() {
    M3 r = zero3();
    for (int i = 0; i < 3; ++i) r.m[i][i] = cx(1.0, 0.0);
    return r;
}
/* nalgebra gemm for 3x3: result column j = sum_k a.col(k) * b[k][j], k ascending */
inline M3 operator*(const M3 &a, const M3 &b) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            Cx s = a.m[i][0] * b.m[0][j];
            s = s + a.m[i][1] * b.m[1][j];
            s = s + a.m[i][2] * b.m[2][j];
            r.m[i][j] = s;
        }
    return r;
}
inline M3 operator+(const M3 &a, const M3 &b) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j];
    return r;
}
inline M3 operator-(const M3 &a, const M3 &b) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j];
    return r;
}
/* matrix * complex scalar (element * scalar) */
inline M3 operator*(const M3 &a, Cx c) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] * c;
    return r;
}
inline M3 adjoint(const M3 &a) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = conj(a.m[j][i]);
    return r;
}
inline Cx trace(const M3 &a) { return a.m[0][0] + a.m[1][1] + a.m[2][2]; }

/* nalgebra 3x3 determinant (cofactor expansion along the first row) */
inline Cx determinant(const M3 &a) {
    const Cx m11 = a.m[0][0], m12 = a.m[0][1], m13 = a.m[0][2];
    const Cx m21 = a.m[1][0], m22 = a.m[1][1], m23 = a.m[1][2];
    const Cx m31 = a.m[2][0], m32 = a.m[2][1], m33 = a.m[2][2];
    const Cx minor_m12_m23 = m22 * m33 - m32 * m23;
    const Cx minor_m11_m23 = m21 * m33 - m31 * m23;
    const Cx minor_m11_m22 = m21 * m32 - m31 * m22;
    return m11 * minor_m12_m23 - m12 * minor_m11_m23 + m13 * minor_m11_m22;
}

/* serde layout <-> M3: 18 doubles, column-major, (re, im) */
inline M3 load_m3(const double *p) {
    M3 r;
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 3; ++row) r.m[row][c] = cx(p[(c * 3 + row) * 2], p[(c * 3 + row) * 2 + 1]);
    return r;
}
inline void store_m3(const M3 &a, double *p) {
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 3; ++row) {
            p[(c * 3 + row) * 2] = a.m[row][c].re;
            p[(c * 3 + row) * 2 + 1] = a.m[row][c].im;
        }
}

/* ---- su(3) generators T^a = lambda^a / 2, src/su3.rs:24-194 ---- */
constexpr double MINUS_ONE_OVER_SQRT_3 = -0.5773502691896258;
constexpr double ONE_OVER_2_SQRT_3 = 0.2886751345948129;

M3 make_generator(int a) {
    M3 g = zero3();
    switch (a) {
    case 0: g.m[0][1] = cx(0.5); g.m[1][0] = cx(0.5); break;
    case 1: g.m[0][1] = cx(0.0, -0.5); g.m[1][0] = cx(0.0, 0.5); break;
    case 2: g.m[0][0] = cx(0.5); g.m[1][1] = cx(-0.5); break;
    case 3: g.m[0][2] = cx(0.5); g.m[2][0] = cx(0.5); break;
    case 4: g.m[0][2] = cx(0.0, -0.5); g.m[2][0] = cx(0.0, 0.5); break;
    case 5: g.m[1][2] = cx(0.5); g.m[2][1] = cx(0.5); break;
    case 6: g.m[1][2] = cx(0.0, -0.5); g.m[2][1] = cx(0.0, 0.5); break;
    default:
        g.m[0][0] = cx(ONE_OVER_2_SQRT_3);
        g.m[1][1] = cx(ONE_OVER_2_SQRT_3);
        g.m[2][2] = cx(MINUS_ONE_OVER_SQRT_3);
        break;
    }
    return g;
}

struct Generators {
    M3 g[8];
    M3 sum; /* GENERATORS.iter().sum(), used by gauss_sum_div (src/field.rs:1212) */
    Generators() {
        M3 s = zero3();
        for (int a = 0; a < 8; ++a) {
            g[a] = make_generator(a);
            s = s + g[a];
        }
        sum = s;
    }
};
const Generators &gens() {
    static const Generators G;
    return G;
}

/* Su3Adjoint::to_matrix, src/field.rs:106-112: sum_a T^a * e^a, folded from zero */
inline M3 to_matrix(const double *e8) {
    const Generators &G = gens();
    M3 r = zero3();
    for (int a = 0; a < 8; ++a) r = r + G.g[a] * cx(e8[a]);
    return r;
}
/* Su3Adjoint::trace_squared, src/field.rs:164-167 */
inline double trace_squared(const double *e8) {
    double s = 0.0;
    for (int a = 0; a < 8; ++a) s = s + e8[a] * e8[a];
    return s / 2.0;
}

/* 1/n! with n! held exactly (u128 in the reference, src/su3.rs:750-775) */
double inv_factorial(int n) {
    unsigned __int128 f = 1;
    for (int i = 2; i <= n; ++i) f *= (unsigned __int128)i;
    return 1.0 / (double)f;
}

/* su3_exp_i, src/su3.rs:832-855 (Cayley-Hamilton, N = 26) */
M3 su3_exp_i(const double *adj) {
    const int N_LOOP = 25;
    const Cx I = cx(0.0, 1.0);
    Cx q0 = cx(inv_factorial(N_LOOP));
    Cx q1 = cx(0.0), q2 = cx(0.0);
    const M3 m = to_matrix(adj);
    const Cx d = determinant(m) * I;
    const Cx t = cx(-0.5 * trace_squared(adj));
    for (int i = N_LOOP - 1; i >= 0; --i) {
        const Cx q0_n = cx(inv_factorial(i)) + d * q2;
        const Cx q1_n = I * (q0 - t * q2);
        const Cx q2_n = I * q1;
        q0 = q0_n;
        q1 = q1_n;
        q2 = q2_n;
    }
    M3 diag = zero3();
    for (int i = 0; i < 3; ++i) diag.m[i][i] = q0;
    return diag + m * q1 + (m * m) * q2;
}

/* su3_exp_r, src/su3.rs:916-938 */
M3 su3_exp_r(const double *adj) {
    const int N_LOOP = 25;
    const Cx I = cx(0.0, 1.0);
    Cx q0 = cx(inv_factorial(N_LOOP));
    Cx q1 = cx(0.0), q2 = cx(0.0);
    const M3 m = to_matrix(adj);
    const Cx d = determinant(m) * I;
    const Cx t = cx(-0.5 * trace_squared(adj));
    for (int i = N_LOOP - 1; i >= 0; --i) {
        const Cx q0_n = cx(inv_factorial(i)) - (I * d) * q2;
        const Cx q1_n = q0 - t * q2;
        const Cx q2_n = q1;
        q0 = q0_n;
        q1 = q1_n;
        q2 = q2_n;
    }
    M3 diag = zero3();
    for (int i = 0; i < 3; ++i) diag.m[i][i] = q0;
    return diag + m * q1 + (m * m) * q2;
}

/* ---- vectors for Gram-Schmidt, src/su3.rs:279-309 ---- */
struct V3 {
    Cx v[3];
};
inline double norm(const V3 &a) {
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s = s + modulus_squared(a.v[i]);
    return std::sqrt(s);
}
/* nalgebra try_normalize(eps): None when the norm <= eps */
inline bool try_normalize(const V3 &a, double eps, V3 &out) {
    const double n = norm(a);
    if (n <= eps) return false;
    for (int i = 0; i < 3; ++i) out.v[i] = cx(a.v[i].re / n, a.v[i].im / n);
    return true;
}
/* non-conjugating dot: sum_i a_i * b_i */
inline Cx dot(const V3 &a, const V3 &b) {
    Cx s = a.v[0] * b.v[0];
    s = s + a.v[1] * b.v[1];
    s = s + a.v[2] * b.v[2];
    return s;
}
inline V3 conjv(const V3 &a) {
    V3 r;
    for (int i = 0; i < 3; ++i) r.v[i] = conj(a.v[i]);
    return r;
}
inline V3 cross(const V3 &a, const V3 &b) {
    V3 r;
    r.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
    r.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
    r.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
    return r;
}
/* create_matrix_from_2_vector, src/su3.rs:279-287: columns [v1, v2, conj(v1) x conj(v2)] */
M3 create_matrix_from_2_vector(const V3 &v1, const V3 &v2) {
    const V3 c = cross(conjv(v1), conjv(v2));
    M3 r;
    for (int i = 0; i < 3; ++i) {
        r.m[i][0] = v1.v[i];
        r.m[i][1] = v2.v[i];
        r.m[i][2] = c.v[i];
    }
    return r;
}
/* ortho_matrix_from_2_vector, src/su3.rs:290-295 */
M3 ortho_matrix_from_2_vector(const V3 &v1, const V3 &v2) {
    V3 v1_new;
    if (!try_normalize(v1, F64_EPS, v1_new)) v1_new = v1;
    const Cx proj = dot(conjv(v1_new), v2);
    V3 v2_temp;
    for (int i = 0; i < 3; ++i) v2_temp.v[i] = v2.v[i] - v1_new.v[i] * proj;
    V3 v2_new;
    if (!try_normalize(v2_temp, F64_EPS, v2_new)) v2_new = v2_temp;
    return create_matrix_from_2_vector(v1_new, v2_new);
}
/* orthonormalize_matrix, src/su3.rs:298-303 */
M3 orthonormalize_matrix(const M3 &m) {
    V3 v1, v2;
    for (int i = 0; i < 3; ++i) {
        v1.v[i] = m.m[i][0];
        v2.v[i] = m.m[i][1];
    }
    return ortho_matrix_from_2_vector(v1, v2);
}

/* ---- random numbers ---- */
struct Rng {
    uint64_t s[4];
    bool has_spare = false;
    double spare = 0.0;
};
inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
uint64_t splitmix64(uint64_t &x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
uint64_t next_u64(Rng &r) {
    const uint64_t result = rotl(r.s[0] + r.s[3], 23) + r.s[0];
    const uint64_t t = r.s[1] << 17;
    r.s[2] ^= r.s[0];
    r.s[3] ^= r.s[1];
    r.s[1] ^= r.s[2];
    r.s[0] ^= r.s[3];
    r.s[2] ^= t;
    r.s[3] = rotl(r.s[3], 45);
    return result;
}
/* rand 0.8 UniformFloat<f64>: 52 random mantissa bits in [1,2), minus 1, * scale + low */
double uniform(Rng &r, double low, double high) {
    double scale = high - low;
    const double max_rand = 1.0 - F64_EPS; /* largest value0_1 = 1 - 2^-52 */
    while (scale * max_rand + low >= high) scale = std::nextafter(scale, 0.0);
    const uint64_t bits = (next_u64(r) >> 12) | 0x3FF0000000000000ULL;
    double value1_2;
    std::memcpy(&value1_2, &bits, sizeof(double));
    const double value0_1 = value1_2 - 1.0;
    return value0_1 * scale + low;
}
double standard_normal(Rng &r) {
    if (r.has_spare) {
        r.has_spare = false;
        return r.spare;
    }
    /* Box-Muller: u1 in (0,1], u2 in [0,1) */
    const double u1 = 1.0 - uniform(r, 0.0, 1.0);
    const double u2 = uniform(r, 0.0, 1.0);
    const double rad = std::sqrt(-2.0 * std::log(u1));
    const double ang = 2.0 * M_PI * u2;
    r.spare = rad * std::sin(ang);
    r.has_spare = true;
    return rad * std::cos(ang);
}

/* random_su3 / rand_su3_with_dis, src/su3.rs:322-355 */
V3 random_vec_3(Rng &r) {
    V3 v;
    for (int i = 0; i < 3; ++i) {
        const double re = uniform(r, -1.0, 1.0);
        const double im = uniform(r, -1.0, 1.0);
        v.v[i] = cx(re, im);
    }
    return v;
}
M3 random_su3(Rng &r) {
    V3 v1 = random_vec_3(r);
    while (norm(v1) <= F64_EPS) v1 = random_vec_3(r);
    V3 v2 = random_vec_3(r);
    while (modulus(dot(v1, v2)) <= F64_EPS) v2 = random_vec_3(r);
    return ortho_matrix_from_2_vector(v1, v2);
}

/* ---- lattice geometry, src/lattice.rs ---- */
struct Lattice {
    int D;
    long L;
    long V;
    long pw[5];
    Lattice(int d, long l) : D(d), L(l) {
        pw[0] = 1;
        for (int i = 1; i <= 4; ++i) pw[i] = pw[i - 1] * (i <= d ? l : 1);
        V = pw[d];
    }
    /* LatticePoint::to_index, src/lattice.rs:909-916 */
    long index(const long *x) const {
        long s = 0;
        for (int i = 0; i < D; ++i) s += (x[i] % L) * pw[i];
        return s;
    }
    void coords(long site, long *x) const {
        for (int i = 0; i < D; ++i) x[i] = (site / pw[i]) % L;
    }
    /* add_point_direction_n with n = 1, src/lattice.rs:303-323 */
    long neighbour(long site, int mu, bool positive) const {
        long x[4] = {0, 0, 0, 0};
        coords(site, x);
        if (positive) {
            x[mu] = (x[mu] + 1) % L;
        } else {
            if (x[mu] < 1) x[mu] = L - (1 - x[mu]);
            else x[mu] = (x[mu] - 1) % L;
        }
        return index(x);
    }
};

/* a signed direction: index + sign */
struct Dir {
    int index;
    bool positive;
};

/* LinkMatrix::matrix, src/field.rs:726-740: U_{-mu}(x) = U_mu(x - mu)^dagger */
inline M3 link_matrix(const Lattice &lat, const double *links, long site, Dir d) {
    if (d.positive) return load_m3(links + (site * lat.D + d.index) * 18);
    const long s = lat.neighbour(site, d.index, false);
    return adjoint(load_m3(links + (s * lat.D + d.index) * 18));
}
inline long add_dir(const Lattice &lat, long site, Dir d) { return lat.neighbour(site, d.index, d.positive); }

/* sij, src/field.rs:743-758: S_ij(x) = U_j(x) U_i(x+j) U_j(x+i)^dagger */
inline M3 sij(const Lattice &lat, const double *links, long site, Dir di, Dir dj) {
    const M3 u_j = link_matrix(lat, links, site, dj);
    const long p_j = add_dir(lat, site, dj);
    const M3 u_i_p_j = link_matrix(lat, links, p_j, di);
    const long p_i = add_dir(lat, site, di);
    const M3 u_j_pi_d = adjoint(link_matrix(lat, links, p_i, dj));
    return (u_j * u_i_p_j) * u_j_pi_d;
}
/* pij, src/field.rs:761-771: P_ij(x) = U_i(x) S_ij(x)^dagger */
inline M3 pij(const Lattice &lat, const double *links, long site, Dir di, Dir dj) {
    const M3 s = sij(lat, links, site, di, dj);
    const M3 u_i = link_matrix(lat, links, site, di);
    return u_i * adjoint(s);
}

/* clover, src/field.rs:806-820: C_ij = P_ij + P_{j,-i} + P_{-i,-j} + P_{-j,i} */
inline M3 clover(const Lattice &lat, const double *links, long site, Dir di, Dir dj) {
    const Dir mi{di.index, !di.positive}, mj{dj.index, !dj.positive};
    return ((pij(lat, links, site, di, dj) + pij(lat, links, site, dj, mi)) + pij(lat, links, site, mi, mj)) +
           pij(lat, links, site, mj, di);
}
/* complex division as num-complex divides: (a + ib) / (c + id) = ((ac + bd) + i(bc - ad)) / (c^2 + d^2) */
inline M3 div_cx(const M3 &m, Cx c) {
    const double n = c.re * c.re + c.im * c.im;
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const Cx a = m.m[i][j];
            r.m[i][j] = Cx{(a.re * c.re + a.im * c.im) / n, (a.im * c.re - a.re * c.im) / n};
        }
    return r;
}
/* f_mu_nu, src/field.rs:822-835: (C_ij - C_ji) / (8 size^2) */
inline M3 f_mu_nu(const Lattice &lat, double size, const double *links, long site, Dir di, Dir dj) {
    const M3 m = clover(lat, links, site, di, dj) - clover(lat, links, site, dj, di);
    return div_cx(m, cx(8.0 * size * size));
}
/* levi_civita, src/utils.rs:306-318: product over i > j of sign(index[i] - index[j]) */
inline int levi_civita3(int a, int b, int c) {
    auto sg = [](int x, int y) { return x > y ? 1 : (x < y ? -1 : 0); };
    return sg(b, a) * sg(c, a) * sg(c, b);
}
/* magnetic_field, src/field.rs:849-871: sum_i sum_j eps(k, i, j) F_ij / (2i), positive directions */
inline M3 magnetic_field(const Lattice &lat, double size, const double *links, long site, int k) {
    M3 sum = zero3();
    for (int i = 0; i < lat.D; ++i) {
        M3 inner = zero3();
        for (int j = 0; j < lat.D; ++j) {
            const M3 f = f_mu_nu(lat, size, links, site, Dir{i, true}, Dir{j, true});
            inner = inner + f * cx((double)levi_civita3(k, i, j));
        }
        sum = sum + inner;
    }
    return div_cx(sum, Cx{0.0, 2.0});
}

/* Direction::directions(): [+0, -0, +1, -1, ...], procedural_macro/src/lib.rs:53-83 */
inline Dir direction_at(int k) { return Dir{k / 2, (k % 2) == 0}; }

/* derivative_e at one site, src/simulation/state.rs:1420-1448 */
void derivative_e_site(const Lattice &lat, const double *links, double size, long site, double *out /*D*8*/) {
    const Generators &G = gens();
    const double c = -std::sqrt(2.0 / 3.0);
    for (int mu = 0; mu < lat.D; ++mu) {
        const Dir dir{mu, true};
        const M3 u_i = link_matrix(lat, links, site, dir);
        M3 sum_s = zero3();
        for (int k = 0; k < 2 * lat.D; ++k) {
            const Dir d2 = direction_at(k);
            if (d2.index == mu) continue;
            sum_s = sum_s + adjoint(sij(lat, links, site, dir, d2));
        }
        for (int a = 0; a < 8; ++a) out[mu * 8 + a] = c * trace((G.g[a] * u_i) * sum_s).im / size;
    }
}

/* derivative_u for one link, src/simulation/state.rs:1407-1417 */
inline M3 derivative_u_link(const Lattice &lat, const double *links, const double *efield, double size, long site,
                            int mu) {
    const Cx c = cx(0.0, std::sqrt(2.0 * 3.0));
    const M3 u_i = link_matrix(lat, links, site, Dir{mu, true});
    const M3 e_i = to_matrix(efield + (site * lat.D + mu) * 8);
    return ((e_i * u_i) * c) * cx(1.0 / size);
}

/* EField::gauss, src/field.rs:1174-1195 */
M3 gauss_site(const Lattice &lat, const double *links, const double *efield, long site) {
    M3 sum = zero3();
    for (int mu = 0; mu < lat.D; ++mu) {
        const M3 e_i = to_matrix(efield + (site * lat.D + mu) * 8);
        const M3 u_mi = link_matrix(lat, links, site, Dir{mu, false});
        const long p_mi = lat.neighbour(site, mu, false);
        const M3 e_m_i = to_matrix(efield + (p_mi * lat.D + mu) * 8);
        sum = sum + (e_i - (u_mi * e_m_i) * adjoint(u_mi));
    }
    return sum;
}

/* EField::gauss_sum_div, src/field.rs:1199-1220 */
double gauss_sum_div(const Lattice &lat, const double *links, const double *efield) {
    const M3 gsum = gens().sum;
    double total = 0.0;
#pragma omp parallel for reduction(+ : total) schedule(static)
    for (long site = 0; site < lat.V; ++site) {
        const M3 g = gauss_site(lat, links, efield, site);
        total += modulus(trace(gsum * g));
    }
    return total;
}

/* EField::project_to_gauss_step, src/field.rs:1301-1337 */
void project_to_gauss_step(const Lattice &lat, const double *links, const double *e_in, double *e_out) {
    const Generators &G = gens();
    const Cx K = cx(0.12, 0.0);
#pragma omp parallel for schedule(static)
    for (long site = 0; site < lat.V; ++site) {
        for (int mu = 0; mu < lat.D; ++mu) {
            const M3 u = link_matrix(lat, links, site, Dir{mu, true});
            const M3 gauss = gauss_site(lat, links, e_in, site);
            const M3 gauss_p = gauss_site(lat, links, e_in, lat.neighbour(site, mu, true));
            const M3 inner = ((((u * gauss) * adjoint(u)) * gauss_p) - gauss) * K;
            const double *e = e_in + (site * lat.D + mu) * 8;
            for (int a = 0; a < 8; ++a) {
                const M3 term = inner + G.g[a] * cx(e[a]);
                e_out[(site * lat.D + mu) * 8 + a] = 2.0 * trace(G.g[a] * term).re;
            }
        }
    }
}

/* EField::project_to_gauss, src/field.rs:1265-1294.  max_steps caps the loop (the
 * reference has no cap); steps counts project_to_gauss_step calls (1 + 4k). */
int project_to_gauss(const Lattice &lat, const double *links, const double *e_in, std::vector<double> &out,
                     int max_steps, int *steps) {
    const size_t n = (size_t)lat.V * lat.D * 8;
    std::vector<double> cur(n), nxt(n);
    project_to_gauss_step(lat, links, e_in, cur.data());
    int done = 1;
    const double threshold = F64_EPS * (double)(lat.V * 4 * 8 * 10);
    for (;;) {
        const double val_dif = gauss_sum_div(lat, links, cur.data());
        if (std::isnan(val_dif)) {
            if (steps) *steps = done;
            return OR_ERR_GAUSS_PROJECTION;
        }
        if (val_dif <= threshold) break;
        if (max_steps > 0 && done + 4 > max_steps) {
            if (steps) *steps = done;
            return OR_ERR_NOT_CONVERGED;
        }
        for (int k = 0; k < 4; ++k) {
            project_to_gauss_step(lat, links, cur.data(), nxt.data());
            cur.swap(nxt);
            ++done;
        }
    }
    out.swap(cur);
    if (steps) *steps = done;
    return OR_OK;
}

/* hamiltonian_links, src/simulation/state.rs:821-849 */
double hamiltonian_links(const Lattice &lat, const double *links, double beta) {
    double total = 0.0;
#pragma omp parallel for reduction(+ : total) schedule(static)
    for (long site = 0; site < lat.V; ++site) {
        double s_site = 0.0;
        for (int i = 0; i < lat.D; ++i) {
            double s_i = 0.0;
            for (int j = i + 1; j < lat.D; ++j) {
                const M3 p = pij(lat, links, site, Dir{i, true}, Dir{j, true});
                s_i = s_i + (1.0 - trace(p).re / 3.0);
            }
            s_site = s_site + s_i;
        }
        total += s_site;
    }
    return total * beta;
}

/* hamiltonian_efield, src/simulation/state.rs:1370-1385 */
double hamiltonian_efield(const Lattice &lat, const double *efield, double beta) {
    double total = 0.0;
#pragma omp parallel for reduction(+ : total) schedule(static)
    for (long site = 0; site < lat.V; ++site) {
        double s = 0.0;
        for (int mu = 0; mu < lat.D; ++mu) s = s + trace_squared(efield + (site * lat.D + mu) * 8);
        total += s;
    }
    return total * beta;
}

/* SymplecticEulerRayon::link_matrix_integrate + integrate_link,
 * src/integrator/symplectic_euler_rayon.rs:65-81, src/integrator/mod.rs:216-233.
 * A new buffer per call, as in the reference. */
std::vector<double> link_matrix_integrate(const Lattice &lat, const double *links, const double *efield, double size,
                                          double dt) {
    std::vector<double> out((size_t)lat.V * lat.D * 18);
#pragma omp parallel for schedule(static)
    for (long site = 0; site < lat.V; ++site) {
        for (int mu = 0; mu < lat.D; ++mu) {
            const M3 init = load_m3(links + (site * lat.D + mu) * 18);
            const M3 du = derivative_u_link(lat, links, efield, size, site, mu);
            store_m3(init + du * cx(dt), out.data() + (site * lat.D + mu) * 18);
        }
    }
    return out;
}

/* SymplecticEulerRayon::e_field_integrate + integrate_efield,
 * src/integrator/symplectic_euler_rayon.rs:88-104, src/integrator/mod.rs:240-254 */
std::vector<double> e_field_integrate(const Lattice &lat, const double *links, const double *efield, double size,
                                      double dt) {
    std::vector<double> out((size_t)lat.V * lat.D * 8);
#pragma omp parallel for schedule(static)
    for (long site = 0; site < lat.V; ++site) {
        double deriv[4 * 8];
        derivative_e_site(lat, links, size, site, deriv);
        for (int mu = 0; mu < lat.D; ++mu)
            for (int a = 0; a < 8; ++a) {
                const size_t k = ((size_t)site * lat.D + mu) * 8 + a;
                out[k] = efield[k] + deriv[mu * 8 + a] * dt;
            }
    }
    return out;
}

/* Link update by the exponential instead of the first-order step: U' = exp(i c E) U with
 * c = dt sqrt(2 C_A) / size, the exponential from su3_exp_i (src/su3.rs:832-855).  The reference
 * has su3_exp_i but no integrator that applies it; this is the variant the device integrator
 * offers, and it is checked link by link against this restatement. */
std::vector<double> link_matrix_integrate_exp(const Lattice &lat, const double *links, const double *efield, double size,
                                              double dt, bool normalize) {
    std::vector<double> out((size_t)lat.V * lat.D * 18);
    const double c = dt * std::sqrt(2.0 * 3.0) / size;
#pragma omp parallel for schedule(static)
    for (long site = 0; site < lat.V; ++site) {
        for (int mu = 0; mu < lat.D; ++mu) {
            double v[8];
            for (int a = 0; a < 8; ++a) v[a] = c * efield[(site * lat.D + mu) * 8 + a];
            M3 u = su3_exp_i(v) * load_m3(links + (site * lat.D + mu) * 18);
            if (normalize) u = orthonormalize_matrix(u);
            store_m3(u, out.data() + (site * lat.D + mu) * 18);
        }
    }
    return out;
}

struct Fields {
    std::vector<double> links, efield;
};

/* SymplecticIntegrator for SymplecticEulerRayon, src/integrator/symplectic_euler_rayon.rs:120-252 */
Fields integrate_once(const Lattice &lat, const Fields &in, double size, int mode, double dt) {
    Fields out;
    switch (mode) {
    case OR_SYNC_SYNC:
        out.links = link_matrix_integrate(lat, in.links.data(), in.efield.data(), size, dt);
        out.efield = e_field_integrate(lat, in.links.data(), in.efield.data(), size, dt);
        break;
    case OR_LEAP_LEAP:
        out.links = link_matrix_integrate(lat, in.links.data(), in.efield.data(), size, dt);
        out.efield = e_field_integrate(lat, out.links.data(), in.efield.data(), size, dt);
        break;
    case OR_SYNC_LEAP:
        out.efield = e_field_integrate(lat, in.links.data(), in.efield.data(), size, dt / 2.0);
        out.links = in.links;
        break;
    case OR_LEAP_SYNC:
        out.links = link_matrix_integrate(lat, in.links.data(), in.efield.data(), size, dt);
        out.efield = e_field_integrate(lat, out.links.data(), in.efield.data(), size, dt / 2.0);
        break;
    case OR_SYMPLECTIC_EXP:
    case OR_SYMPLECTIC_EXP_NORMALIZE: {
        const std::vector<double> e_half = e_field_integrate(lat, in.links.data(), in.efield.data(), size, dt / 2.0);
        out.links = link_matrix_integrate_exp(lat, in.links.data(), e_half.data(), size, dt,
                                              mode == OR_SYMPLECTIC_EXP_NORMALIZE);
        out.efield = e_field_integrate(lat, out.links.data(), e_half.data(), size, dt / 2.0);
        break;
    }
    default: { /* OR_SYMPLECTIC */
        const std::vector<double> e_half = e_field_integrate(lat, in.links.data(), in.efield.data(), size, dt / 2.0);
        out.links = link_matrix_integrate(lat, in.links.data(), e_half.data(), size, dt);
        out.efield = e_field_integrate(lat, out.links.data(), e_half.data(), size, dt / 2.0);
        break;
    }
    }
    return out;
}

/* ---- Monte Carlo sweeps: MetropolisHastingsSweep and HeatBathSweep
 * (src/simulation/monte_carlo/metropolis_hastings_sweep.rs, heat_bath.rs), per link as the reference
 * updates it, in checkerboard order (for each direction mu, all links (x, mu) with sum_i x_i even,
 * then odd: links of one class share no staple, so the class can be updated at once) with random
 * numbers from a Philox4x32-10 stream per link (the device's stream; the reference's rand streams
 * are not restated). */

/* Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11) */
struct U4 {
    uint32_t x, y, z, w;
};
inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        c = U4{(uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0};
    }
    return c;
}
/* uniforms in [0, 1) with 53 bits from counter blocks (link, sweep lo, sweep hi, 0x80000000 + call) */
struct LinkRng {
    uint32_t k0, k1, link, s_lo, s_hi;
    uint32_t call = 0;
    double buf = 0.0;
    bool has = false;
    static double u01(uint32_t hi, uint32_t lo) {
        return (double)((((uint64_t)hi << 32) | lo) >> 11) * (1.0 / 9007199254740992.0);
    }
    double next() {
        if (has) {
            has = false;
            return buf;
        }
        const U4 r = philox4x32_10(U4{link, s_lo, s_hi, 0x80000000u + call++}, k0, k1);
        buf = u01(r.z, r.w);
        has = true;
        return u01(r.x, r.y);
    }
    double uniform(double a, double b) { return a + (b - a) * next(); } /* Uniform::new(a, b) */
    double open_closed01() { return 1.0 - next(); }                    /* OpenClosed01 */
    bool half() { return next() < 0.5; }                               /* Bernoulli(0.5) */
};

constexpr int kMaxRedraws = 10000; /* bound of every rejection loop (the reference loops without one) */

struct M2 {
    Cx m[2][2];
};
inline M2 mul2(const M2 &a, const M2 &b) {
    M2 r;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j];
    return r;
}
inline M2 adj2(const M2 &a) {
    M2 r;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) r.m[i][j] = conj(a.m[j][i]);
    return r;
}
/* su2::complex_matrix_from_vec (src/su2.rs:134-140): x0 1 + sum_i PAULI_MATRICES[i] (i x_i), with the
 * reference's constants PAULI_1 = [[0,1],[1,0]], PAULI_2 = [[0,-i],[i,0]], PAULI_3 = [[1,0],[0,1]]
 * (src/su2.rs:13-49: PAULI_3 is written as the identity) */
inline M2 complex_matrix_from_vec(double x0, const double *x) {
    static const Cx P[3][2][2] = {{{{0, 0}, {1, 0}}, {{1, 0}, {0, 0}}},
                                  {{{0, 0}, {0, -1}}, {{0, 1}, {0, 0}}},
                                  {{{1, 0}, {0, 0}}, {{0, 0}, {1, 0}}}};
    M2 r;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            Cx t = cx(0.0, 0.0);
            for (int k = 0; k < 3; ++k) t = t + P[k][i][j] * Cx{0.0, x[k]};
            r.m[i][j] = Cx{i == j ? 1.0 : 0.0, 0.0} * Cx{x0, 0.0} + t;
        }
    return r;
}
/* su2::random_su2_close_to_unity (src/su2.rs:80-100) */
inline M2 random_su2_close_to_unity(double spread, LinkRng &rng) {
    double r[3];
    for (double &v : r) v = rng.uniform(-1.0, 1.0);
    const double n = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    double x[3];
    for (int i = 0; i < 3; ++i) x[i] = (n > F64_EPS ? r[i] / n : r[i]) * spread;
    const double x0u = std::sqrt(1.0 - (x[0] * x[0] + x[1] * x[1] + x[2] * x[2]));
    const double x0 = rng.half() ? x0u : -x0u;
    return complex_matrix_from_vec(x0, x);
}
/* su2::random_su2 (src/su2.rs:200-216) */
inline M2 random_su2(LinkRng &rng) {
    Cx v[2];
    double n = 0.0;
    for (int tries = 0; tries < kMaxRedraws; ++tries) {
        for (Cx &c : v) {
            const double re = rng.uniform(-1.0, 1.0);
            c = Cx{re, rng.uniform(-1.0, 1.0)};
        }
        n = std::sqrt(modulus_squared(v[0]) + modulus_squared(v[1]));
        if (std::isnormal(n)) break;
    }
    const Cx d{n, 0.0};
    auto divc = [&](Cx a) { /* num-complex division by (n, 0) */
        const double q = d.re * d.re + d.im * d.im;
        return Cx{(a.re * d.re + a.im * d.im) / q, (a.im * d.re - a.re * d.im) / q};
    };
    const Cx a = divc(v[0]), b = divc(v[1]);
    M2 r;
    r.m[0][0] = a;
    r.m[0][1] = b;
    r.m[1][0] = Cx{-b.re, b.im}; /* -conj(b) */
    r.m[1][1] = conj(a);
    return r;
}
/* su3::get_r / get_s / get_t (src/su3.rs:428-530): SU(2) blocks embedded at (0,1), (0,2), (1,2) */
inline M3 embed(const M2 &m, int p, int q) {
    M3 r = identity3();
    r.m[p][p] = m.m[0][0];
    r.m[p][q] = m.m[0][1];
    r.m[q][p] = m.m[1][0];
    r.m[q][q] = m.m[1][1];
    return r;
}
/* su3::get_su2_*_unorm (src/su3.rs:559-659): su2::project_to_su2_unorm(m) = m - m^dag + 1 conj(Tr m)
 * of the sub-block */
inline M2 su2_unorm(const M3 &in, int p, int q) {
    M2 b;
    b.m[0][0] = in.m[p][p];
    b.m[0][1] = in.m[p][q];
    b.m[1][0] = in.m[q][p];
    b.m[1][1] = in.m[q][q];
    const Cx tr = conj(b.m[0][0] + b.m[1][1]);
    M2 r;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) r.m[i][j] = (b.m[i][j] - conj(b.m[j][i])) + Cx{i == j ? 1.0 : 0.0, 0.0} * tr;
    return r;
}
/* su3::random_su3_close_to_unity (src/su3.rs:385-398) */
inline M3 random_su3_close_to_unity(double spread, LinkRng &rng) {
    const M3 r = embed(random_su2_close_to_unity(spread, rng), 0, 1);
    const M3 s = embed(random_su2_close_to_unity(spread, rng), 0, 2);
    const M3 t = embed(random_su2_close_to_unity(spread, rng), 1, 2);
    M3 x = (r * s) * t;
    if (rng.half()) x = adjoint(x);
    return x;
}
/* statistics::ModifiedNormal, HeatBathDistributionNorm, HeatBathDistribution
 * (src/statistics/distribution.rs:76-101, :320-350, :199-218) */
inline double modified_normal(double param, LinkRng &rng) {
    double r[3];
    for (double &v : r) v = rng.open_closed01();
    const double c = std::cos(2.0 * 3.141592653589793 * r[1]);
    return std::sqrt(-(std::log(r[0]) + c * c * std::log(r[2])) / (2.0 * param));
}
inline double heat_bath_norm(double param, LinkRng &rng) {
    for (int tries = 0; tries < kMaxRedraws; ++tries) {
        const double r = rng.uniform(0.0, 1.0);
        const double lambda = modified_normal(param, rng);
        if (r * r <= 1.0 - lambda * lambda) return 1.0 - 2.0 * lambda * lambda;
    }
    return 1.0;
}
inline M2 heat_bath_sample(double param, LinkRng &rng) {
    const double x0 = heat_bath_norm(param, rng);
    double x[3], n = 0.0;
    for (int tries = 0; tries < kMaxRedraws; ++tries) {
        for (double &v : x) v = rng.uniform(-1.0, 1.0);
        n = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        if (n > F64_EPS) break;
    }
    const double f = std::sqrt(1.0 - x0 * x0);
    for (double &v : x) v = v / n * f;
    return complex_matrix_from_vec(x0, x);
}
/* HeatBathSweep::heat_bath_su2 (src/simulation/monte_carlo/heat_bath.rs:71-86) */
inline M2 heat_bath_su2(const M2 &staple, double beta, LinkRng &rng) {
    const Cx det = staple.m[0][0] * staple.m[1][1] - staple.m[1][0] * staple.m[0][1];
    const double k = std::sqrt(det.re);
    if (std::isnormal(k)) {
        const M2 a = adj2(staple);
        M2 v;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) {
                const Cx z = a.m[i][j];
                const double q = k * k;
                v.m[i][j] = Cx{(z.re * k) / q, (z.im * k) / q};
            }
        return mul2(heat_bath_sample(beta * k, rng), v);
    }
    return random_su2(rng);
}
/* the staple of the Monte Carlo methods (src/simulation/monte_carlo/mod.rs:339-362):
 * sum over nu != mu of S_mu,nu(x)^dag + U_{-nu}(x+mu) U_mu(x-nu)^dag U_nu(x-nu) */
inline M3 mc_staple(const Lattice &lat, const double *links, long site, int mu) {
    M3 sum = zero3();
    for (int nu = 0; nu < lat.D; ++nu) {
        if (nu == mu) continue;
        const M3 el1 = adjoint(sij(lat, links, site, Dir{mu, true}, Dir{nu, true}));
        const long xpmu = lat.neighbour(site, mu, true);
        const M3 u1 = link_matrix(lat, links, xpmu, Dir{nu, false});
        const long xmnu = lat.neighbour(site, nu, false);
        const M3 u2 = adjoint(link_matrix(lat, links, xmnu, Dir{mu, true}));
        const M3 u3 = link_matrix(lat, links, xmnu, Dir{nu, true});
        sum = sum + (el1 + (u1 * u2) * u3);
    }
    return sum;
}
inline long parity_of(const Lattice &lat, long site) {
    long x[4], p = 0;
    lat.coords(site, x);
    for (int i = 0; i < lat.D; ++i) p += x[i];
    return p & 1;
}

bool supported_dim(int dim) { return dim >= 2 && dim <= 4; }

int check_lattice(int dim, long L) {
    if (dim == 0) return OR_ERR_ZERO_DIMENSION;
    if (!supported_dim(dim)) return OR_ERR_UNSUPPORTED_D;
    if (L < 2) return OR_ERR_DIM_TOO_SMALL;
    return OR_OK;
}

/* ---- overrelaxation (src/simulation/monte_carlo/overrelaxation.rs) ----
 * Both methods use the singular value decomposition a = U S V^dag of a = staple^dag (nalgebra's
 * SVD, not vendored).  Restated from the eigen-decomposition of the Hermitian a^dag a = V S^2 V^dag
 * by cyclic complex Jacobi rotations (Golub & Van Loan, Matrix Computations, section 8.5; the phase
 * of the off-diagonal element is removed first, then the real rotation with
 * tan 2 theta = 2 |h_pq| / (h_qq - h_pp)), 5 sweeps over the pairs (0,1), (0,2), (1,2), and
 * U = a V S^-1.  Cyclic Jacobi converges quadratically: on random staples and on staples with
 * singular values 1e-9 apart, 4 sweeps already give the updates of 8 to 2e-15; the fifth is margin.  For distinct singular values both updates are independent of the SVD's phase and
 * ordering freedom (a diagonal phase or a permutation commutes through `reverse`), so they are the
 * reference's values.  The device evaluates the same operations in the same order without fused
 * multiply-adds (the update divides by the smallest singular value, so it magnifies rounding
 * differences; identical arithmetic keeps FP64 parity at 1e-12):
 *   rotation (:92-104): rot = U V^dag, U' = rot U^dag rot
 *   reverse  (:160-172): U' = U reverse(U^dag L V) V^dag, reverse negating the off-diagonal entries
 *                        (su3.rs:705-714)
 */
void herm3_eigen_jacobi(M3 h, double lam[3], M3 &v) {
    v = identity3();
    const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 5; ++sweep)
        for (const auto &pq : pairs) {
            const int p = pq[0], q = pq[1];
            /* sqrt of the sum of squares, not hypot, so that the device can evaluate it identically */
            const double c = std::sqrt(h.m[p][q].re * h.m[p][q].re + h.m[p][q].im * h.m[p][q].im);
            if (!(c > 0.0)) continue;
            const Cx ph = cx(h.m[p][q].re / c, h.m[p][q].im / c); /* e^{i phi} */
            const double tau = (h.m[q][q].re - h.m[p][p].re) / (2.0 * c);
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
            const double cs = 1.0 / std::sqrt(1.0 + t * t), sn = t * cs;
            /* J = identity except J_pp = cs, J_pq = sn, J_qp = -sn e^{-i phi}, J_qq = cs e^{-i phi} */
            M3 j = identity3();
            j.m[p][p] = cx(cs);
            j.m[p][q] = cx(sn);
            j.m[q][p] = conj(ph) * cx(-sn);
            j.m[q][q] = conj(ph) * cx(cs);
            h = (adjoint(j) * h) * j;
            v = v * j;
        }
    for (int k = 0; k < 3; ++k) lam[k] = h.m[k][k].re;
}
/* U and V of a = U S V^dag, S from the eigenvalues of a^dag a */
void svd3(const M3 &a, M3 &u, M3 &v) {
    double lam[3];
    herm3_eigen_jacobi(adjoint(a) * a, lam, v);
    const M3 av = a * v;
    for (int k = 0; k < 3; ++k) {
        const double s = std::sqrt(std::fmax(lam[k], 0.0));
        for (int i = 0; i < 3; ++i) u.m[i][k] = cx(av.m[i][k].re / s, av.m[i][k].im / s);
    }
}
M3 reverse3(const M3 &x) {
    M3 r = x;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (i != j) r.m[i][j] = cx(-x.m[i][j].re, -x.m[i][j].im);
    return r;
}
M3 overrelax_link(const M3 &link, const M3 &staple, int method) {
    M3 u, v;
    svd3(adjoint(staple), u, v);
    if (method == 0) {
        const M3 rot = u * adjoint(v);
        return (rot * adjoint(link)) * rot;
    }
    return (u * reverse3((adjoint(u) * link) * v)) * adjoint(v);
}

} // namespace

/* ======================= C interface ======================= */

extern "C" {

void *or_rng_new(uint64_t seed) {
    Rng *r = new Rng();
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) r->s[i] = splitmix64(x);
    return r;
}
void or_rng_free(void *rng) { delete static_cast<Rng *>(rng); }
uint64_t or_rng_next_u64(void *rng) { return next_u64(*static_cast<Rng *>(rng)); }
double or_rng_uniform(void *rng, double low, double high) { return uniform(*static_cast<Rng *>(rng), low, high); }
double or_rng_standard_normal(void *rng) { return standard_normal(*static_cast<Rng *>(rng)); }

/* LatticeCyclic::new, src/lattice.rs:190-201 (checks in the same order) */
int or_lattice_new(int dim, double size, long number_of_points) {
    if (dim == 0) return OR_ERR_ZERO_DIMENSION;
    if (size <= 0.0 || std::isnan(size) || std::isinf(size)) return OR_ERR_NON_POSITIVE_SIZE;
    if (number_of_points < 2) return OR_ERR_DIM_TOO_SMALL;
    if (!supported_dim(dim)) return OR_ERR_UNSUPPORTED_D;
    return OR_OK;
}

void or_generators(double *out) {
    for (int a = 0; a < 8; ++a) store_m3(gens().g[a], out + 18 * a);
}
void or_su3_to_matrix(const double *adj8, double *out18) { store_m3(to_matrix(adj8), out18); }
void or_su3_exp_i(const double *adj8, double *out18) { store_m3(su3_exp_i(adj8), out18); }
void or_su3_exp_r(const double *adj8, double *out18) { store_m3(su3_exp_r(adj8), out18); }
void or_orthonormalize(const double *m18, double *out18) { store_m3(orthonormalize_matrix(load_m3(m18)), out18); }
void or_random_su3(void *rng, double *out18) { store_m3(random_su3(*static_cast<Rng *>(rng)), out18); }
void or_matmul(const double *a18, const double *b18, double *out18) { store_m3(load_m3(a18) * load_m3(b18), out18); }
void or_determinant(const double *m18, double *out2) {
    const Cx d = determinant(load_m3(m18));
    out2[0] = d.re;
    out2[1] = d.im;
}

/* LinkMatrix::new_determinist, src/field.rs:646-659: one random_su3 per link, link order */
int or_links_random(int dim, int L, void *rng, double *links) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
    Rng &r = *static_cast<Rng *>(rng);
    for (long k = 0; k < lat.V * dim; ++k) store_m3(random_su3(r), links + k * 18);
    return OR_OK;
}
/* LinkMatrix::new_cold, src/field.rs:703-707 */
int or_links_cold(int dim, int L, double *links) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
    for (long k = 0; k < lat.V * dim; ++k) store_m3(identity3(), links + k * 18);
    return OR_OK;
}
/* EField::new_determinist, src/field.rs:1086-1099: site order, then mu, then a */
int or_efield_normal(int dim, int L, void *rng, double std_dev, double *efield) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    if (!(std_dev >= 0.0) || std::isinf(std_dev)) return OR_ERR_INVALID_NORMAL;
    const Lattice lat(dim, L);
    Rng &r = *static_cast<Rng *>(rng);
    for (long k = 0; k < lat.V * dim * 8; ++k) efield[k] = 0.0 + std_dev * standard_normal(r);
    return OR_OK;
}

int or_hamiltonian_links(int dim, int L, double beta, const double *links, double *out) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    *out = hamiltonian_links(Lattice(dim, L), links, beta);
    return OR_OK;
}
int or_hamiltonian_efield(int dim, int L, double beta, const double *efield, double *out) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    *out = hamiltonian_efield(Lattice(dim, L), efield, beta);
    return OR_OK;
}
/* LinkMatrix::average_trace_plaquette, src/field.rs:775-804 */
int or_average_trace_plaquette(int dim, int L, const double *links, double *re, double *im) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
    double sre = 0.0, sim = 0.0;
#pragma omp parallel for reduction(+ : sre, sim) schedule(static)
    for (long site = 0; site < lat.V; ++site) {
        Cx s_site = cx(0.0);
        for (int i = 0; i < dim; ++i) {
            Cx s_i = cx(0.0);
            for (int j = i + 1; j < dim; ++j) s_i = s_i + trace(pij(lat, links, site, Dir{i, true}, Dir{j, true}));
            s_site = s_site + s_i;
        }
        sre += s_site.re;
        sim += s_site.im;
    }
    const double n_plaq = (double)(lat.V * ((dim * (dim - 1)) / 2));
    *re = sre / n_plaq;
    *im = sim / n_plaq;
    return OR_OK;
}
/* clover / f_mu_nu / magnetic_field at one point (signed directions: index, positive flag) */
int or_clover(int dim, int L, const double *links, long site, int i, int i_pos, int j, int j_pos, double *out18) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
    if (site < 0 || site >= lat.V || i < 0 || i >= dim || j < 0 || j >= dim) return OR_ERR_INVALID_ARGUMENT;
    store_m3(clover(lat, links, site, Dir{i, i_pos != 0}, Dir{j, j_pos != 0}), out18);
    return OR_OK;
}
int or_f_mu_nu(int dim, int L, double size, const double *links, long site, int i, int j, double *out18) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
    if (site < 0 || site >= lat.V || i < 0 || i >= dim || j < 0 || j >= dim) return OR_ERR_INVALID_ARGUMENT;
    store_m3(f_mu_nu(lat, size, links, site, Dir{i, true}, Dir{j, true}), out18);
    return OR_OK;
}
int or_magnetic_field(int dim, int L, double size, const double *links, long site, int k, double *out18) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
    if (site < 0 || site >= lat.V || k < 0 || k >= dim) return OR_ERR_INVALID_ARGUMENT;
    store_m3(magnetic_field(lat, size, links, site, k), out18);
    return OR_OK;
}
/* MetropolisHastingsSweep::next_element (metropolis_hastings_sweep.rs:147-177) in checkerboard
 * order; link (site, mu) draws from LinkRng(seed, link = site * D + mu, sweep) */
int or_metropolis_sweep(int dim, int L, double beta, const double *links_in, int n_update, double spread,
                        uint64_t seed, uint64_t sweep, double *links_out, long *n_accepted, double *prob_sum) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    if (L % 2 != 0 || n_update <= 0 || !(spread > 0.0) || !(spread < 1.0)) return OR_ERR_INVALID_ARGUMENT;
    const Lattice lat(dim, L);
    std::memcpy(links_out, links_in, sizeof(double) * 18 * lat.V * dim);
    long acc = 0;
    double psum = 0.0;
    for (int mu = 0; mu < dim; ++mu)
        for (long parity = 0; parity < 2; ++parity)
            for (long site = 0; site < lat.V; ++site) {
                if (parity_of(lat, site) != parity) continue;
                LinkRng rng{(uint32_t)seed, (uint32_t)(seed >> 32), (uint32_t)(site * dim + mu), (uint32_t)sweep,
                            (uint32_t)(sweep >> 32)};
                double *lp = links_out + (site * dim + mu) * 18;
                const M3 old_m = load_m3(lp);
                M3 new_m = old_m;
                for (int k = 0; k < n_update; ++k)
                    new_m = orthonormalize_matrix(random_su3_close_to_unity(spread, rng)) * new_m;
                const M3 a = mc_staple(lat, links_out, site, mu);
                const double ds = -trace((new_m - old_m) * a).re * beta / 3.0;
                const double p = std::fmax(std::fmin(std::exp(-ds), 1.0), 0.0);
                psum += p;
                if (p >= 1.0 || rng.next() < p) {
                    store_m3(new_m, lp);
                    ++acc;
                }
            }
    if (n_accepted) *n_accepted = acc;
    if (prob_sum) *prob_sum = psum;
    return OR_OK;
}
/* HeatBathSweep::next_element (heat_bath.rs:88-121) in checkerboard order */
int or_heat_bath_sweep(int dim, int L, double beta, const double *links_in, uint64_t seed, uint64_t sweep,
                       double *links_out) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    if (L % 2 != 0 || !(beta > 0.0)) return OR_ERR_INVALID_ARGUMENT;
    const Lattice lat(dim, L);
    std::memcpy(links_out, links_in, sizeof(double) * 18 * lat.V * dim);
    for (int mu = 0; mu < dim; ++mu)
        for (long parity = 0; parity < 2; ++parity)
            for (long site = 0; site < lat.V; ++site) {
                if (parity_of(lat, site) != parity) continue;
                LinkRng rng{(uint32_t)seed, (uint32_t)(seed >> 32), (uint32_t)(site * dim + mu), (uint32_t)sweep,
                            (uint32_t)(sweep >> 32)};
                double *lp = links_out + (site * dim + mu) * 18;
                const M3 u = load_m3(lp);
                const M3 a = mc_staple(lat, links_out, site, mu);
                const M3 r = embed(heat_bath_su2(su2_unorm(u * a, 0, 1), beta, rng), 0, 1);
                const M3 s = embed(heat_bath_su2(su2_unorm((r * u) * a, 0, 2), beta, rng), 0, 2);
                const M3 t = embed(heat_bath_su2(su2_unorm(((s * r) * u) * a, 1, 2), beta, rng), 1, 2);
                store_m3(((t * s) * r) * u, lp);
            }
    return OR_OK;
}
/* OverrelaxationSweepRotation (method 0) / OverrelaxationSweepReverse (1) in checkerboard order:
 * for each mu, the links (x, mu) with even, then odd sum of coordinates (the device order; the
 * reference updates one link after another in lattice order) */
int or_overrelaxation_sweep(int dim, int L, const double *links_in, int method, double *links_out) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    if (L % 2 != 0 || (method != 0 && method != 1)) return OR_ERR_INVALID_ARGUMENT;
    const Lattice lat(dim, L);
    std::memcpy(links_out, links_in, sizeof(double) * 18 * lat.V * dim);
    for (int mu = 0; mu < dim; ++mu)
        for (long parity = 0; parity < 2; ++parity)
            for (long site = 0; site < lat.V; ++site) {
                if (parity_of(lat, site) != parity) continue;
                double *lp = links_out + (site * dim + mu) * 18;
                store_m3(overrelax_link(load_m3(lp), mc_staple(lat, links_out, site, mu), method), lp);
            }
    return OR_OK;
}
/* one link's update from its link and staple matrices (18 doubles each, reference layout) */
int or_overrelax_link(const double *link18, const double *staple18, int method, double *out18) {
    if (method != 0 && method != 1) return OR_ERR_INVALID_ARGUMENT;
    store_m3(overrelax_link(load_m3(link18), load_m3(staple18), method), out18);
    return OR_OK;
}

int or_gauss(int dim, int L, const double *links, const double *efield, long site, double *out18) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
    if (site < 0 || site >= lat.V) return OR_ERR_INVALID_ARGUMENT;
    store_m3(gauss_site(lat, links, efield, site), out18);
    return OR_OK;
}
int or_gauss_sum_div(int dim, int L, const double *links, const double *efield, double *out) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    *out = gauss_sum_div(Lattice(dim, L), links, efield);
    return OR_OK;
}
int or_project_to_gauss(int dim, int L, const double *links, const double *efield_in, double *efield_out,
                        int max_steps, int *steps_done) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
    std::vector<double> out;
    const int rc = project_to_gauss(lat, links, efield_in, out, max_steps, steps_done);
    if (rc) return rc;
    std::memcpy(efield_out, out.data(), out.size() * sizeof(double));
    return OR_OK;
}
/* LinkMatrix::normalize, src/field.rs:897-901 */
int or_normalize(int dim, int L, double *links) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < lat.V * dim; ++k) store_m3(orthonormalize_matrix(load_m3(links + k * 18)), links + k * 18);
    return OR_OK;
}
int or_derivative_e(int dim, int L, double size, const double *links, double *force) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
#pragma omp parallel for schedule(static)
    for (long site = 0; site < lat.V; ++site) derivative_e_site(lat, links, size, site, force + site * dim * 8);
    return OR_OK;
}
int or_derivative_u(int dim, int L, double size, const double *links, const double *efield, double *du) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const Lattice lat(dim, L);
#pragma omp parallel for schedule(static)
    for (long site = 0; site < lat.V; ++site)
        for (int mu = 0; mu < dim; ++mu)
            store_m3(derivative_u_link(lat, links, efield, size, site, mu), du + (site * dim + mu) * 18);
    return OR_OK;
}

/* simulate_{sync,leap,symplectic}_n, src/simulation/state.rs:399-491 and :603-647 */
int or_integrate(int dim, int L, double size, const double *links_in, const double *efield_in, int mode, double dt,
                 int n, double *links_out, double *efield_out) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    if (n <= 0) return OR_ERR_ZERO_INTEGRATION;
    if (mode < OR_SYNC_SYNC || mode > OR_SYMPLECTIC_EXP_NORMALIZE) return OR_ERR_INVALID_ARGUMENT;
    const Lattice lat(dim, L);
    Fields f;
    f.links.assign(links_in, links_in + (size_t)lat.V * dim * 18);
    f.efield.assign(efield_in, efield_in + (size_t)lat.V * dim * 8);
    for (int i = 0; i < n; ++i) f = integrate_once(lat, f, size, mode, dt);
    std::memcpy(links_out, f.links.data(), f.links.size() * sizeof(double));
    std::memcpy(efield_out, f.efield.data(), f.efield.size() * sizeof(double));
    return OR_OK;
}

/* simulate_using_leapfrog_n, src/simulation/state.rs:318-357 */
int or_leapfrog_n(int dim, int L, double size, const double *links_in, const double *efield_in, double dt, int n,
                  double *links_out, double *efield_out) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    if (n <= 0) return OR_ERR_ZERO_INTEGRATION;
    const Lattice lat(dim, L);
    Fields f;
    f.links.assign(links_in, links_in + (size_t)lat.V * dim * 18);
    f.efield.assign(efield_in, efield_in + (size_t)lat.V * dim * 8);
    f = integrate_once(lat, f, size, OR_SYNC_LEAP, dt);
    for (int i = 1; i < n; ++i) f = integrate_once(lat, f, size, OR_LEAP_LEAP, dt);
    f = integrate_once(lat, f, size, OR_LEAP_SYNC, dt);
    std::memcpy(links_out, f.links.data(), f.links.size() * sizeof(double));
    std::memcpy(efield_out, f.efield.data(), f.efield.size() * sizeof(double));
    return OR_OK;
}

/* HybridMonteCarloDiagnostic::next_element with injected randomness,
 * src/simulation/monte_carlo/hybrid_monte_carlo.rs:465-471 and :573-613 */
int or_hmc_trajectory(int dim, int L, double size, double beta, const double *links_in, const double *efield_raw,
                      double dt, int n_steps, double uniform_draw, int max_gauss_steps, double *links_out,
                      double *efield_out, int *accepted, double *prob, double *h_old, double *h_new,
                      int *gauss_steps) {
    const int st = check_lattice(dim, L);
    if (st) return st;
    const double std_dev = 0.5 / beta; /* Normal(0, 0.5/beta) must be a valid distribution */
    if (!(std_dev >= 0.0) || std::isinf(std_dev)) return OR_ERR_INVALID_NORMAL;
    if (n_steps <= 0) return OR_ERR_ZERO_INTEGRATION;
    const Lattice lat(dim, L);
    /* new_random_e_state: project the drawn field, src/simulation/state.rs:1093-1108 */
    std::vector<double> e_proj;
    const int rc = project_to_gauss(lat, links_in, efield_raw, e_proj, max_gauss_steps, gauss_steps);
    if (rc) return rc;
    Fields f0;
    f0.links.assign(links_in, links_in + (size_t)lat.V * dim * 18);
    f0.efield = e_proj;
    Fields f = f0;
    for (int i = 0; i < n_steps; ++i) f = integrate_once(lat, f, size, OR_SYMPLECTIC, dt);
    /* probability_of_replacement, hybrid_monte_carlo.rs:584-589 */
    const double h0 = hamiltonian_links(lat, f0.links.data(), beta) + hamiltonian_efield(lat, f0.efield.data(), beta);
    const double h1 = hamiltonian_links(lat, f.links.data(), beta) + hamiltonian_efield(lat, f.efield.data(), beta);
    double p = std::fmax(std::fmin(std::exp(h0 - h1), 1.0), 0.0);
    p = std::fmax(std::fmin(p, 1.0), 0.0);
    /* rand 0.8 Bernoulli: p == 1 is always true, otherwise u < p */
    const bool acc = (p >= 1.0) || (uniform_draw < p);
    const Fields &res = acc ? f : f0;
    std::memcpy(links_out, res.links.data(), res.links.size() * sizeof(double));
    if (efield_out) std::memcpy(efield_out, res.efield.data(), res.efield.size() * sizeof(double));
    *accepted = acc ? 1 : 0;
    *prob = p;
    *h_old = h0;
    *h_new = h1;
    return OR_OK;
}

void or_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}
int or_get_threads(void) { return omp_get_max_threads(); }

} /* extern "C" */
