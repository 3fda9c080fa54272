// su3.cuh -- 3x3 complex matrix arithmetic for the device (CUDA cores, FMA chains).
//
// SU(3) products are 3x3 complex contractions (27 complex multiply-adds): too small and
// too irregular for tensor cores, so they run as FMA chains in registers, templated on
// the storage/compute type T (double or float).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

// Index checks (builds with -DLQ_BOUNDS_CHECK=1, the stand-in for a memory checker): the site and
// plane indices the kernels form (neighbours, coordinates, tile planes) are compared with their
// bounds; a bad one is counted in this translation unit's g_bounds, replaced by 0 so that the access
// stays inside the array, and reported through lq_bounds_check.  Off by default: no cost.
#ifndef LQ_BOUNDS_CHECK
#define LQ_BOUNDS_CHECK 0
#endif

namespace lq {

// host side: every translation unit of a checked build registers the reader of its own counters
// (lq_api.cu keeps the list)
int register_bounds_reader(int (*read)(unsigned long long *count, unsigned long long *first, int reset));
#if LQ_BOUNDS_CHECK
// [0] bad indices seen, [1] the first one (value + 1; plane indices as (nplanes << 32) | plane)
static __device__ unsigned long long g_bounds[2];
__device__ __forceinline__ void bounds_fail(unsigned long long v) {
    if (atomicAdd(&g_bounds[0], 1ull) == 0ull) g_bounds[1] = v + 1ull;
}
static int read_bounds(unsigned long long *count, unsigned long long *first, int reset) {
    unsigned long long h[2] = {0ull, 0ull};
    cudaError_t e = cudaMemcpyFromSymbol(h, g_bounds, sizeof(h));
    if (e == cudaSuccess && reset) {
        const unsigned long long z[2] = {0ull, 0ull};
        e = cudaMemcpyToSymbol(g_bounds, z, sizeof(z));
    }
    if (e != cudaSuccess) return (int)e;
    *count += h[0];
    if (h[0] && !*first) *first = h[1];
    return 0;
}
[[maybe_unused]] static const int g_bounds_registered = register_bounds_reader(read_bounds);
#endif
// site index < n, else counted (checked builds) and replaced by 0
__device__ __forceinline__ uint32_t checked_site(uint32_t site, uint32_t n) {
#if LQ_BOUNDS_CHECK
    if (site >= n) {
        bounds_fail(site);
        return 0u;
    }
#else
    (void)n;
#endif
    return site;
}

template <typename T> struct cpx {
    T re, im;
};

// 3x3 complex matrix, row-major e[row*3 + col]
template <typename T> struct mat3 {
    cpx<T> e[9];
};

template <typename T> struct vec2_t;
template <> struct vec2_t<double> { using type = double2; };
template <> struct vec2_t<float> { using type = float2; };

// su(3) generator constants of T^8 (src/su3.rs:176-180)
constexpr double kOneOver2Sqrt3 = 0.2886751345948129;
constexpr double kMinusOneOverSqrt3 = -0.5773502691896258;

template <typename T> __device__ __forceinline__ cpx<T> cmk(T r, T i) { return cpx<T>{r, i}; }

template <typename T> __device__ __forceinline__ void mat_zero(mat3<T> &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) m.e[k] = cmk<T>(T(0), T(0));
}

template <typename T> __device__ __forceinline__ void mat_identity(mat3<T> &m) {
    mat_zero(m);
    m.e[0].re = T(1);
    m.e[4].re = T(1);
    m.e[8].re = T(1);
}

// r = a * b
template <typename T> __device__ __forceinline__ void mul_nn(const mat3<T> &a, const mat3<T> &b, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T re = a.e[i * 3].re * b.e[j].re;
            T im = a.e[i * 3].re * b.e[j].im;
            re = fma(-a.e[i * 3].im, b.e[j].im, re);
            im = fma(a.e[i * 3].im, b.e[j].re, im);
#pragma unroll
            for (int k = 1; k < 3; ++k) {
                re = fma(a.e[i * 3 + k].re, b.e[k * 3 + j].re, re);
                re = fma(-a.e[i * 3 + k].im, b.e[k * 3 + j].im, re);
                im = fma(a.e[i * 3 + k].re, b.e[k * 3 + j].im, im);
                im = fma(a.e[i * 3 + k].im, b.e[k * 3 + j].re, im);
            }
            r.e[i * 3 + j] = cmk(re, im);
        }
}

// One complex multiply-add term of mul_nn, with AR / BR telling that a / b is known to be real
// (the diagonal of a Hermitian matrix, whose imaginary part is an exact zero): the multiply-adds
// with that zero are left out.  fma(x, 0, y) returns y, so every nonzero result rounds as the
// full term rounds it (only the sign of an exact zero can differ).
//   cmul_first: re = a.re b.re - a.im b.im, im = a.re b.im + a.im b.re (mul_nn's k = 0 term)
//   cmul_acc  : re += a.re b.re - a.im b.im, im += a.re b.im + a.im b.re, in mul_nn's order
template <bool AR, bool BR, typename T>
__device__ __forceinline__ void cmul_first(const cpx<T> &a, const cpx<T> &b, T &re, T &im) {
    if constexpr (AR && BR) {
        re = a.re * b.re;
        im = T(0);
    } else if constexpr (AR) {
        re = a.re * b.re;
        im = a.re * b.im;
    } else if constexpr (BR) {
        re = a.re * b.re;
        im = a.im * b.re;
    } else {
        re = a.re * b.re;
        im = a.re * b.im;
        re = fma(-a.im, b.im, re);
        im = fma(a.im, b.re, im);
    }
}
template <bool AR, bool BR, typename T>
__device__ __forceinline__ void cmul_acc(const cpx<T> &a, const cpx<T> &b, T &re, T &im) {
    re = fma(a.re, b.re, re);
    if constexpr (!AR && !BR) re = fma(-a.im, b.im, re);
    if constexpr (!BR) im = fma(a.re, b.im, im);
    if constexpr (!AR) im = fma(a.im, b.re, im);
}

// r = a * g for g Hermitian with a real diagonal (as herm_load builds it): mul_nn less the 18
// multiply-adds with the zero imaginary parts of g's diagonal.
template <typename T> __device__ __forceinline__ void mul_nh(const mat3<T> &a, const mat3<T> &g, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T re, im;
            if (j == 0) cmul_first<false, true>(a.e[i * 3], g.e[j], re, im);
            else cmul_first<false, false>(a.e[i * 3], g.e[j], re, im);
            if (j == 1) cmul_acc<false, true>(a.e[i * 3 + 1], g.e[3 + j], re, im);
            else cmul_acc<false, false>(a.e[i * 3 + 1], g.e[3 + j], re, im);
            if (j == 2) cmul_acc<false, true>(a.e[i * 3 + 2], g.e[6 + j], re, im);
            else cmul_acc<false, false>(a.e[i * 3 + 2], g.e[6 + j], re, im);
            r.e[i * 3 + j] = cmk(re, im);
        }
}

// r = a * b^dagger
template <typename T> __device__ __forceinline__ void mul_na(const mat3<T> &a, const mat3<T> &b, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            // sum_k a[i][k] * conj(b[j][k])
            T re = a.e[i * 3].re * b.e[j * 3].re;
            T im = -a.e[i * 3].re * b.e[j * 3].im;
            re = fma(a.e[i * 3].im, b.e[j * 3].im, re);
            im = fma(a.e[i * 3].im, b.e[j * 3].re, im);
#pragma unroll
            for (int k = 1; k < 3; ++k) {
                re = fma(a.e[i * 3 + k].re, b.e[j * 3 + k].re, re);
                re = fma(a.e[i * 3 + k].im, b.e[j * 3 + k].im, re);
                im = fma(-a.e[i * 3 + k].re, b.e[j * 3 + k].im, im);
                im = fma(a.e[i * 3 + k].im, b.e[j * 3 + k].re, im);
            }
            r.e[i * 3 + j] = cmk(re, im);
        }
}

// r = a^dagger * b
template <typename T> __device__ __forceinline__ void mul_an(const mat3<T> &a, const mat3<T> &b, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            // sum_k conj(a[k][i]) * b[k][j]
            T re = a.e[i].re * b.e[j].re;
            T im = a.e[i].re * b.e[j].im;
            re = fma(a.e[i].im, b.e[j].im, re);
            im = fma(-a.e[i].im, b.e[j].re, im);
#pragma unroll
            for (int k = 1; k < 3; ++k) {
                re = fma(a.e[k * 3 + i].re, b.e[k * 3 + j].re, re);
                re = fma(a.e[k * 3 + i].im, b.e[k * 3 + j].im, re);
                im = fma(a.e[k * 3 + i].re, b.e[k * 3 + j].im, im);
                im = fma(-a.e[k * 3 + i].im, b.e[k * 3 + j].re, im);
            }
            r.e[i * 3 + j] = cmk(re, im);
        }
}

// r = a * b^dagger for a product known to be Hermitian (u G u^dag with G Hermitian): the upper
// triangle is computed as mul_na computes it, the diagonal's real part likewise (its imaginary part
// is zero), and the lower triangle is the conjugate of the upper one -- 54 multiply-adds, not 108.
template <typename T> __device__ __forceinline__ void mul_na_herm(const mat3<T> &a, const mat3<T> &b, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T d = a.e[i * 3].re * b.e[i * 3].re;
        d = fma(a.e[i * 3].im, b.e[i * 3].im, d);
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            d = fma(a.e[i * 3 + k].re, b.e[i * 3 + k].re, d);
            d = fma(a.e[i * 3 + k].im, b.e[i * 3 + k].im, d);
        }
        r.e[i * 4] = cmk(d, T(0));
#pragma unroll
        for (int j = i + 1; j < 3; ++j) {
            T re = a.e[i * 3].re * b.e[j * 3].re;
            T im = -a.e[i * 3].re * b.e[j * 3].im;
            re = fma(a.e[i * 3].im, b.e[j * 3].im, re);
            im = fma(a.e[i * 3].im, b.e[j * 3].re, im);
#pragma unroll
            for (int k = 1; k < 3; ++k) {
                re = fma(a.e[i * 3 + k].re, b.e[j * 3 + k].re, re);
                re = fma(a.e[i * 3 + k].im, b.e[j * 3 + k].im, re);
                im = fma(-a.e[i * 3 + k].re, b.e[j * 3 + k].im, im);
                im = fma(a.e[i * 3 + k].im, b.e[j * 3 + k].re, im);
            }
            r.e[i * 3 + j] = cmk(re, im);
            r.e[j * 3 + i] = cmk(re, -im);
        }
    }
}

// r = a^dagger * b for a product known to be Hermitian (U^dag E U): as mul_na_herm
template <typename T> __device__ __forceinline__ void mul_an_herm(const mat3<T> &a, const mat3<T> &b, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T d = a.e[i].re * b.e[i].re;
        d = fma(a.e[i].im, b.e[i].im, d);
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            d = fma(a.e[k * 3 + i].re, b.e[k * 3 + i].re, d);
            d = fma(a.e[k * 3 + i].im, b.e[k * 3 + i].im, d);
        }
        r.e[i * 4] = cmk(d, T(0));
#pragma unroll
        for (int j = i + 1; j < 3; ++j) {
            T re = a.e[i].re * b.e[j].re;
            T im = a.e[i].re * b.e[j].im;
            re = fma(a.e[i].im, b.e[j].im, re);
            im = fma(-a.e[i].im, b.e[j].re, im);
#pragma unroll
            for (int k = 1; k < 3; ++k) {
                re = fma(a.e[k * 3 + i].re, b.e[k * 3 + j].re, re);
                re = fma(a.e[k * 3 + i].im, b.e[k * 3 + j].im, re);
                im = fma(a.e[k * 3 + i].re, b.e[k * 3 + j].im, im);
                im = fma(-a.e[k * 3 + i].im, b.e[k * 3 + j].re, im);
            }
            r.e[i * 3 + j] = cmk(re, im);
            r.e[j * 3 + i] = cmk(re, -im);
        }
    }
}

// r += a * b^dagger
template <typename T> __device__ __forceinline__ void mul_na_acc(const mat3<T> &a, const mat3<T> &b, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T re = r.e[i * 3 + j].re, im = r.e[i * 3 + j].im;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                re = fma(a.e[i * 3 + k].re, b.e[j * 3 + k].re, re);
                re = fma(a.e[i * 3 + k].im, b.e[j * 3 + k].im, re);
                im = fma(-a.e[i * 3 + k].re, b.e[j * 3 + k].im, im);
                im = fma(a.e[i * 3 + k].im, b.e[j * 3 + k].re, im);
            }
            r.e[i * 3 + j] = cmk(re, im);
        }
}

// r += a^dagger * b
template <typename T> __device__ __forceinline__ void mul_an_acc(const mat3<T> &a, const mat3<T> &b, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T re = r.e[i * 3 + j].re, im = r.e[i * 3 + j].im;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                re = fma(a.e[k * 3 + i].re, b.e[k * 3 + j].re, re);
                re = fma(a.e[k * 3 + i].im, b.e[k * 3 + j].im, re);
                im = fma(a.e[k * 3 + i].re, b.e[k * 3 + j].im, im);
                im = fma(-a.e[k * 3 + i].im, b.e[k * 3 + j].re, im);
            }
            r.e[i * 3 + j] = cmk(re, im);
        }
}

// Hermitian traceless matrix sum_a c^a T^a from its 8 coefficients (Su3Adjoint::to_matrix,
// src/field.rs:106-112), generators T^a = lambda^a / 2 (src/su3.rs:24-194).
template <typename T> __device__ __forceinline__ void adjoint_to_matrix(const T *c, mat3<T> &m) {
    const T h = T(0.5);
    const T c8p = T(kOneOver2Sqrt3) * c[7];
    m.e[0] = cmk(h * c[2] + c8p, T(0));
    m.e[4] = cmk(-h * c[2] + c8p, T(0));
    m.e[8] = cmk(T(kMinusOneOverSqrt3) * c[7], T(0));
    m.e[1] = cmk(h * c[0], -h * c[1]);
    m.e[3] = cmk(h * c[0], h * c[1]);
    m.e[2] = cmk(h * c[3], -h * c[4]);
    m.e[6] = cmk(h * c[3], h * c[4]);
    m.e[5] = cmk(h * c[5], -h * c[6]);
    m.e[7] = cmk(h * c[5], h * c[6]);
}

// out^a = 2 Re Tr(T^a X) for a general 3x3 complex X
template <typename T> __device__ __forceinline__ void two_re_tr_generators(const mat3<T> &x, T *out) {
    out[0] = x.e[3].re + x.e[1].re;
    out[1] = x.e[3].im - x.e[1].im;
    out[2] = x.e[0].re - x.e[4].re;
    out[3] = x.e[6].re + x.e[2].re;
    out[4] = x.e[6].im - x.e[2].im;
    out[5] = x.e[7].re + x.e[5].re;
    out[6] = x.e[7].im - x.e[5].im;
    out[7] = T(2.0 * kOneOver2Sqrt3) * (x.e[0].re + x.e[4].re) + T(2.0 * kMinusOneOverSqrt3) * x.e[8].re;
}

// out^a = Im Tr(T^a X) for a general 3x3 complex X (the projection in derivative_e,
// src/simulation/state.rs:1440)
template <typename T> __device__ __forceinline__ void im_tr_generators(const mat3<T> &x, T *out) {
    const T h = T(0.5);
    out[0] = h * (x.e[3].im + x.e[1].im);
    out[1] = h * (x.e[1].re - x.e[3].re);
    out[2] = h * (x.e[0].im - x.e[4].im);
    out[3] = h * (x.e[6].im + x.e[2].im);
    out[4] = h * (x.e[2].re - x.e[6].re);
    out[5] = h * (x.e[7].im + x.e[5].im);
    out[6] = h * (x.e[5].re - x.e[7].re);
    out[7] = T(kOneOver2Sqrt3) * (x.e[0].im + x.e[4].im) + T(kMinusOneOverSqrt3) * x.e[8].im;
}

// out^a = 2 Re Tr(T^a a b) without forming the full product: the real parts of the diagonal and
// the six off-diagonal entries of a b, in mul_nn's order (90 multiply-adds instead of 108)
template <typename T>
__device__ __forceinline__ void two_re_tr_generators_of_product(const mat3<T> &a, const mat3<T> &b, T *out) {
    auto entry = [&](int i, int j) {
        T re = a.e[i * 3].re * b.e[j].re, im = a.e[i * 3].re * b.e[j].im;
        re = fma(-a.e[i * 3].im, b.e[j].im, re);
        im = fma(a.e[i * 3].im, b.e[j].re, im);
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            re = fma(a.e[i * 3 + k].re, b.e[k * 3 + j].re, re);
            re = fma(-a.e[i * 3 + k].im, b.e[k * 3 + j].im, re);
            im = fma(a.e[i * 3 + k].re, b.e[k * 3 + j].im, im);
            im = fma(a.e[i * 3 + k].im, b.e[k * 3 + j].re, im);
        }
        return cmk(re, im);
    };
    auto diag_re = [&](int i) {
        T re = a.e[i * 3].re * b.e[i].re;
        re = fma(-a.e[i * 3].im, b.e[i].im, re);
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            re = fma(a.e[i * 3 + k].re, b.e[k * 3 + i].re, re);
            re = fma(-a.e[i * 3 + k].im, b.e[k * 3 + i].im, re);
        }
        return re;
    };
    const cpx<T> x1 = entry(0, 1), x3 = entry(1, 0), x2 = entry(0, 2), x6 = entry(2, 0), x5 = entry(1, 2),
                 x7 = entry(2, 1);
    const T x0 = diag_re(0), x4 = diag_re(1), x8 = diag_re(2);
    out[0] = x3.re + x1.re;
    out[1] = x3.im - x1.im;
    out[2] = x0 - x4;
    out[3] = x6.re + x2.re;
    out[4] = x6.im - x2.im;
    out[5] = x7.re + x5.re;
    out[6] = x7.im - x5.im;
    out[7] = T(2.0 * kOneOver2Sqrt3) * (x0 + x4) + T(2.0 * kMinusOneOverSqrt3) * x8;
}

// out^a = 2 Re Tr(T^a a b) for a and b both Hermitian with real diagonals (u G u^dag and G in the
// projection step): two_re_tr_generators_of_product less the 27 multiply-adds with the zero
// imaginary parts of the two diagonals (63 instead of 90).
template <typename T>
__device__ __forceinline__ void two_re_tr_generators_of_hermitian_product(const mat3<T> &a, const mat3<T> &b, T *out) {
    // entry (i, j), i != j, of a b: a's term k is real for k == i, b's for k == j
    auto entry = [&](auto ic, auto jc) {
        constexpr int i = decltype(ic)::value, j = decltype(jc)::value;
        T re, im;
        cmul_first<i == 0, j == 0>(a.e[i * 3], b.e[j], re, im);
        cmul_acc<i == 1, j == 1>(a.e[i * 3 + 1], b.e[3 + j], re, im);
        cmul_acc<i == 2, j == 2>(a.e[i * 3 + 2], b.e[6 + j], re, im);
        return cmk(re, im);
    };
    // real part of the diagonal entry (i, i)
    auto diag_re = [&](auto ic) {
        constexpr int i = decltype(ic)::value;
        T re = a.e[i * 3].re * b.e[i].re;
        if constexpr (i != 0) re = fma(-a.e[i * 3].im, b.e[i].im, re);
        re = fma(a.e[i * 3 + 1].re, b.e[3 + i].re, re);
        if constexpr (i != 1) re = fma(-a.e[i * 3 + 1].im, b.e[3 + i].im, re);
        re = fma(a.e[i * 3 + 2].re, b.e[6 + i].re, re);
        if constexpr (i != 2) re = fma(-a.e[i * 3 + 2].im, b.e[6 + i].im, re);
        return re;
    };
    using I0 = std::integral_constant<int, 0>;
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    const cpx<T> x1 = entry(I0{}, I1{}), x3 = entry(I1{}, I0{}), x2 = entry(I0{}, I2{}), x6 = entry(I2{}, I0{}),
                 x5 = entry(I1{}, I2{}), x7 = entry(I2{}, I1{});
    const T x0 = diag_re(I0{}), x4 = diag_re(I1{}), x8 = diag_re(I2{});
    out[0] = x3.re + x1.re;
    out[1] = x3.im - x1.im;
    out[2] = x0 - x4;
    out[3] = x6.re + x2.re;
    out[4] = x6.im - x2.im;
    out[5] = x7.re + x5.re;
    out[6] = x7.im - x5.im;
    out[7] = T(2.0 * kOneOver2Sqrt3) * (x0 + x4) + T(2.0 * kMinusOneOverSqrt3) * x8;
}

// 1/n! evaluated at compile time
constexpr double inv_factorial(int n) {
    double f = 1.0;
    for (int k = 2; k <= n; ++k) f *= (double)k;
    return 1.0 / f;
}

// exp(i X) - 1 for X = sum_a v^a T^a, by the Cayley-Hamilton recursion of su3_exp_i
// (src/su3.rs:832-855; the method of the OpenQCD su3_fcts notes): exp(i X) = q0 + q1 X + q2 X^2
// with, from q0 = 1/(N-1)!, q1 = q2 = 0 and for i = N-2 down to 0,
//   q0 <- 1/i! + d q2,  q1 <- i (q0 - t q2),  q2 <- i q1,   d = i det X,  t = -Tr(X^2)/2.
// The identity (the 1/0! of the last step) is left out so that a small rotation keeps its
// relative precision.  N = 26 terms as the reference for double; 18 for float, where
// 1/(N-7)! is below the FP32 epsilon (the reference's criterion, src/su3.rs:716-725).
template <typename T> __device__ __forceinline__ void su3_exp_i_minus_one(const T *v, mat3<T> &r) {
    constexpr int NL = (sizeof(T) == 8 ? 26 : 18) - 1;
    mat3<T> m;
    adjoint_to_matrix<T>(v, m);
    // det of the Hermitian X is real: expansion along the first row
    const cpx<T> c0 = cmk(m.e[4].re * m.e[8].re - (m.e[5].re * m.e[5].re + m.e[5].im * m.e[5].im), T(0));
    // m.e[1] * (m.e[3] m.e[8] - m.e[5] m.e[6]) and m.e[2] * (m.e[3] m.e[7] - m.e[4] m.e[6])
    const T a_re = m.e[3].re * m.e[8].re - (m.e[5].re * m.e[6].re - m.e[5].im * m.e[6].im);
    const T a_im = m.e[3].im * m.e[8].re - (m.e[5].re * m.e[6].im + m.e[5].im * m.e[6].re);
    const T b_re = (m.e[3].re * m.e[7].re - m.e[3].im * m.e[7].im) - m.e[4].re * m.e[6].re;
    const T b_im = (m.e[3].re * m.e[7].im + m.e[3].im * m.e[7].re) - m.e[4].re * m.e[6].im;
    const T det = m.e[0].re * c0.re - (m.e[1].re * a_re - m.e[1].im * a_im) + (m.e[2].re * b_re - m.e[2].im * b_im);
    T ts = T(0);
#pragma unroll
    for (int a = 0; a < 8; ++a) ts = fma(v[a], v[a], ts);
    const T t = T(-0.25) * ts; // -Tr(X^2)/2 = -(sum v^2 / 2) / 2
    T inv = T(inv_factorial(NL));
    T q0r = inv, q0i = T(0), q1r = T(0), q1i = T(0), q2r = T(0), q2i = T(0);
#pragma unroll
    for (int i = NL - 1; i >= 0; --i) {
        inv *= T(i + 1);
        const T c = (i == 0) ? T(0) : inv;
        const T n0r = c - det * q2i, n0i = det * q2r;
        const T n1r = -(q0i - t * q2i), n1i = q0r - t * q2r;
        const T n2r = -q1i, n2i = q1r;
        q0r = n0r;
        q0i = n0i;
        q1r = n1r;
        q1i = n1i;
        q2r = n2r;
        q2i = n2i;
    }
    mat3<T> m2;
    mul_nn(m, m, m2);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        T re = q1r * m.e[k].re - q1i * m.e[k].im;
        T im = q1r * m.e[k].im + q1i * m.e[k].re;
        re = fma(q2r, m2.e[k].re, fma(-q2i, m2.e[k].im, re));
        im = fma(q2r, m2.e[k].im, fma(q2i, m2.e[k].re, im));
        r.e[k] = cmk(re, im);
    }
    r.e[0].re += q0r;
    r.e[0].im += q0i;
    r.e[4].re += q0r;
    r.e[4].im += q0i;
    r.e[8].re += q0r;
    r.e[8].im += q0i;
}

// orthonormalize_matrix (src/su3.rs:290-309) in double on a row-major 3x3 (re, im):
// v1 = col0 / |col0|, v2 = col1 - v1 (v1^* . col1), normalised, col2 = conj(v1) x conj(v2);
// a vector whose norm is <= f64::EPSILON is kept unnormalised (try_normalize).
__device__ __forceinline__ void orthonormalize_d(double (&re)[9], double (&im)[9]) {
    double r1[3], i1[3], r2[3], i2[3];
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        r1[row] = re[row * 3];
        i1[row] = im[row * 3];
        r2[row] = re[row * 3 + 1];
        i2[row] = im[row * 3 + 1];
    }
    const double eps = 2.220446049250313e-16;
    const double n1 = sqrt(r1[0] * r1[0] + i1[0] * i1[0] + r1[1] * r1[1] + i1[1] * i1[1] + r1[2] * r1[2] + i1[2] * i1[2]);
    if (n1 > eps) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            r1[k] /= n1;
            i1[k] /= n1;
        }
    }
    double pr = 0.0, pi = 0.0; // sum_k conj(v1_k) v2_k
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        pr += r1[k] * r2[k] + i1[k] * i2[k];
        pi += r1[k] * i2[k] - i1[k] * r2[k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        r2[k] -= r1[k] * pr - i1[k] * pi;
        i2[k] -= r1[k] * pi + i1[k] * pr;
    }
    const double n2 = sqrt(r2[0] * r2[0] + i2[0] * i2[0] + r2[1] * r2[1] + i2[1] * i2[1] + r2[2] * r2[2] + i2[2] * i2[2]);
    if (n2 > eps) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            r2[k] /= n2;
            i2[k] /= n2;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
        // (a x b)_k with a = conj(v1), b = conj(v2)
        const double xr = r1[k1] * r2[k2] - i1[k1] * i2[k2];
        const double xi = -(r1[k1] * i2[k2] + i1[k1] * r2[k2]);
        const double yr = r1[k2] * r2[k1] - i1[k2] * i2[k1];
        const double yi = -(r1[k2] * i2[k1] + i1[k2] * r2[k1]);
        re[k * 3] = r1[k];
        im[k * 3] = i1[k];
        re[k * 3 + 1] = r2[k];
        im[k * 3 + 1] = i2[k];
        re[k * 3 + 2] = xr - yr;
        im[k * 3 + 2] = xi - yi;
    }
}

// ---- tiled structure-of-arrays storage ----
// Sites are grouped in tiles of 32 consecutive sites (one warp).  An array of P planes stores
// plane p of site s at ((s / 32) * P + p) * 32 + s % 32: a warp reads each plane of its tile as
// one contiguous segment.
constexpr int kTile = 32;
__host__ __device__ __forceinline__ size_t tix(uint32_t site, int nplanes, int plane) {
#if LQ_BOUNDS_CHECK && defined(__CUDA_ARCH__)
    if (plane < 0 || plane >= nplanes) {
        bounds_fail(((unsigned long long)(uint32_t)nplanes << 32) | (uint32_t)plane);
        plane = 0;
    }
#endif
    return ((size_t)(site >> 5) * nplanes + plane) * kTile + (site & 31);
}
__host__ __device__ __forceinline__ uint32_t tiles_of(uint32_t V) { return (V + kTile - 1) / kTile; }

// ---- links and momenta inside a tile ----
// Links: entry k of the link of (site, mu) is plane mu*9 + k, a float2 / double2 per site: idx =
// tix(site, P, mu * 9) is entry 0 and entry k lies k * 32 elements further (a warp reads 256 B
// (FP32) or 512 B (FP64) per entry).  Packing FP32 links into float4 pairs of entries was measured
// and not kept: the 128-bit destinations raised the MD kernel's register demand past its
// 96-register budget (spills; 5 % slower at 32^4).
// Momenta: the 8 planes mu*8 .. mu*8+7 of a tile form a block in which the components of one site
// are packed into 16-byte vectors -- FP64: components 2q, 2q+1 = double2 plane q (q = 0..3); FP32:
// components 4q .. 4q+3 = float4 plane q (q = 0, 1) -- so a thread moves its momenta with 4 (FP64)
// or 2 (FP32) 128-bit accesses and a warp touches 512 contiguous bytes per access.  idx =
// tix(site, P, mu * 8) is the site's element of plane 0 in the unpacked form; every array base (an
// allocation, the lo half of a compensated array, an ensemble of a batch, a segment of the
// adjoint's arena) lies whole tiles from a 256-byte aligned allocation, so idx % 32 is the site's
// lane and idx - lane the 16-byte aligned block.

// element offset from idx of entry k of a link
template <typename T> __host__ __device__ __forceinline__ size_t link_off(size_t, int k) { return (size_t)k * kTile; }
// element offset from idx of momentum component a of a link
template <typename T> __host__ __device__ __forceinline__ size_t efield_off(size_t idx, int a) {
    const size_t lane = idx & 31;
    if constexpr (sizeof(T) == 8) return (size_t)(a >> 1) * (2 * kTile) + lane + (a & 1);
    else return (size_t)(a >> 2) * (4 * kTile) + 3 * lane + (a & 3);
}

// one link matrix (read-only path: the arrays read with it are not written by the same launch,
// except by the reading thread itself after its read)
template <typename T> __device__ __forceinline__ void load_link(const typename vec2_t<T>::type *__restrict__ U, size_t idx,
                                                                mat3<T> &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const typename vec2_t<T>::type v = __ldg(U + idx + k * kTile);
        m.e[k] = cmk<T>(v.x, v.y);
    }
}
template <typename T>
__device__ __forceinline__ void store_link(typename vec2_t<T>::type *__restrict__ U, size_t idx, const mat3<T> &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        typename vec2_t<T>::type v;
        v.x = m.e[k].re;
        v.y = m.e[k].im;
        U[idx + k * kTile] = v;
    }
}
// the 8 momentum components of one link (plain loads: momenta are updated in place)
template <typename T> __device__ __forceinline__ void load_efield(const T *E, size_t idx, T (&e)[8]) {
    const size_t lane = idx & 31;
    if constexpr (sizeof(T) == 8) {
        const double2 *q = reinterpret_cast<const double2 *>(E + (idx - lane)) + lane;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const double2 v = q[j * kTile];
            e[2 * j] = v.x;
            e[2 * j + 1] = v.y;
        }
    } else {
        const float4 *q = reinterpret_cast<const float4 *>(E + (idx - lane)) + lane;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float4 v = q[j * kTile];
            e[4 * j] = v.x;
            e[4 * j + 1] = v.y;
            e[4 * j + 2] = v.z;
            e[4 * j + 3] = v.w;
        }
    }
}
template <typename T> __device__ __forceinline__ void store_efield(T *E, size_t idx, const T (&e)[8]) {
    const size_t lane = idx & 31;
    if constexpr (sizeof(T) == 8) {
        double2 *q = reinterpret_cast<double2 *>(E + (idx - lane)) + lane;
#pragma unroll
        for (int j = 0; j < 4; ++j) q[j * kTile] = make_double2(e[2 * j], e[2 * j + 1]);
    } else {
        float4 *q = reinterpret_cast<float4 *>(E + (idx - lane)) + lane;
#pragma unroll
        for (int j = 0; j < 2; ++j) q[j * kTile] = make_float4(e[4 * j], e[4 * j + 1], e[4 * j + 2], e[4 * j + 3]);
    }
}

// w = (sum_a c^a T^a) u for a Hermitian traceless left factor given by its coefficients:
// diagonal entries are real, so each entry of w costs 10 multiply-adds instead of 12.
template <typename T> __device__ __forceinline__ void adj_mul(const T *c, const mat3<T> &u, mat3<T> &w) {
    const T h = T(0.5);
    const T c8p = T(kOneOver2Sqrt3) * c[7];
    const T d[3] = {h * c[2] + c8p, -h * c[2] + c8p, T(kMinusOneOverSqrt3) * c[7]};
    // upper off-diagonal entries e01, e02, e12 (lower ones are their conjugates)
    const cpx<T> e01 = cmk(h * c[0], -h * c[1]), e02 = cmk(h * c[3], -h * c[4]), e12 = cmk(h * c[5], -h * c[6]);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const cpx<T> u0 = u.e[j], u1 = u.e[3 + j], u2 = u.e[6 + j];
        // row 0: d0 u0 + e01 u1 + e02 u2
        T re = d[0] * u0.re, im = d[0] * u0.im;
        re = fma(e01.re, u1.re, re); re = fma(-e01.im, u1.im, re);
        im = fma(e01.re, u1.im, im); im = fma(e01.im, u1.re, im);
        re = fma(e02.re, u2.re, re); re = fma(-e02.im, u2.im, re);
        im = fma(e02.re, u2.im, im); im = fma(e02.im, u2.re, im);
        w.e[j] = cmk(re, im);
        // row 1: conj(e01) u0 + d1 u1 + e12 u2
        re = d[1] * u1.re; im = d[1] * u1.im;
        re = fma(e01.re, u0.re, re); re = fma(e01.im, u0.im, re);
        im = fma(e01.re, u0.im, im); im = fma(-e01.im, u0.re, im);
        re = fma(e12.re, u2.re, re); re = fma(-e12.im, u2.im, re);
        im = fma(e12.re, u2.im, im); im = fma(e12.im, u2.re, im);
        w.e[3 + j] = cmk(re, im);
        // row 2: conj(e02) u0 + conj(e12) u1 + d2 u2
        re = d[2] * u2.re; im = d[2] * u2.im;
        re = fma(e02.re, u0.re, re); re = fma(e02.im, u0.im, re);
        im = fma(e02.re, u0.im, im); im = fma(-e02.im, u0.re, im);
        re = fma(e12.re, u1.re, re); re = fma(e12.im, u1.im, re);
        im = fma(e12.re, u1.im, im); im = fma(-e12.im, u1.re, im);
        w.e[6 + j] = cmk(re, im);
    }
}

// out^a = Im Tr(T^a a b) without forming the full product: only the imaginary parts of the
// diagonal and the six off-diagonal entries of a b enter (90 multiply-adds instead of 108).
// out^a = Im Tr(T^a M) from the entries of M it needs: the off-diagonal pairs and the imaginary
// parts of the diagonal
template <typename T, bool HALF>
__device__ __forceinline__ void im_tr_combine(const cpx<T> &m01, const cpx<T> &m10, const cpx<T> &m02,
                                              const cpx<T> &m20, const cpx<T> &m12, const cpx<T> &m21, T i00, T i11,
                                              T i22, T *out) {
    if constexpr (HALF) {
        const T h = T(0.5);
        out[0] = h * (m10.im + m01.im);
        out[1] = h * (m01.re - m10.re);
        out[2] = h * (i00 - i11);
        out[3] = h * (m20.im + m02.im);
        out[4] = h * (m02.re - m20.re);
        out[5] = h * (m21.im + m12.im);
        out[6] = h * (m12.re - m21.re);
        out[7] = T(kOneOver2Sqrt3) * (i00 + i11) + T(kMinusOneOverSqrt3) * i22;
    } else {
        out[0] = m10.im + m01.im;
        out[1] = m01.re - m10.re;
        out[2] = i00 - i11;
        out[3] = m20.im + m02.im;
        out[4] = m02.re - m20.re;
        out[5] = m21.im + m12.im;
        out[6] = m12.re - m21.re;
        out[7] = T(2.0 * kOneOver2Sqrt3) * (i00 + i11) + T(2.0 * kMinusOneOverSqrt3) * i22;
    }
}

// (HALF = false: twice the value, the factor 1/2 left to the caller -- a power of two, so applying it
// later to a sum of such terms rounds exactly as applying it to each)
template <typename T, bool HALF = true>
__device__ __forceinline__ void im_tr_generators_of_product(const mat3<T> &a, const mat3<T> &b, T *out) {
    auto entry = [&](int i, int j) {
        T re = a.e[i * 3].re * b.e[j].re, im = a.e[i * 3].re * b.e[j].im;
        re = fma(-a.e[i * 3].im, b.e[j].im, re);
        im = fma(a.e[i * 3].im, b.e[j].re, im);
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            re = fma(a.e[i * 3 + k].re, b.e[k * 3 + j].re, re);
            re = fma(-a.e[i * 3 + k].im, b.e[k * 3 + j].im, re);
            im = fma(a.e[i * 3 + k].re, b.e[k * 3 + j].im, im);
            im = fma(a.e[i * 3 + k].im, b.e[k * 3 + j].re, im);
        }
        return cmk(re, im);
    };
    auto diag_im = [&](int i) {
        T im = a.e[i * 3].re * b.e[i].im;
        im = fma(a.e[i * 3].im, b.e[i].re, im);
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            im = fma(a.e[i * 3 + k].re, b.e[k * 3 + i].im, im);
            im = fma(a.e[i * 3 + k].im, b.e[k * 3 + i].re, im);
        }
        return im;
    };
    const cpx<T> m01 = entry(0, 1), m10 = entry(1, 0), m02 = entry(0, 2), m20 = entry(2, 0), m12 = entry(1, 2),
                 m21 = entry(2, 1);
    const T i00 = diag_im(0), i11 = diag_im(1), i22 = diag_im(2);
    im_tr_combine<T, HALF>(m01, m10, m02, m20, m12, m21, i00, i11, i22, out);
}

// acc^a += k out^a, out^a = 2 Re Tr(T^a X Y) for traceless Hermitian X = x^c T^c, Y = y^d T^d from
// their components: out^a = (1/2) d_acd x^c y^d, where Tr(T^a T^c T^d) = (d_acd + i f_acd) / 4 and the symmetric constants of
// SU(3) in the Gell-Mann basis (adjoint_to_matrix's) are d_118 = d_228 = d_338 = -d_888 = 1/sqrt(3),
// d_448 = d_558 = d_668 = d_778 = -1/(2 sqrt(3)), d_146 = d_157 = d_256 = d_344 = d_355 = 1/2,
// d_247 = d_366 = d_377 = -1/2 (1-based indices; 58 multiply-adds instead of the matrix route's ~110)
template <typename T>
__device__ __forceinline__ void two_re_tr_generators_of_traceless_product(const T *x, const T *y, T k, T *acc) {
    // acc^a += k out^a; the constants carry k (q = k/4, r = k/(2 sqrt(3)), s = k/(4 sqrt(3)))
    const T q = k * T(0.25), r = k * T(kOneOver2Sqrt3), s = k * T(0.5 * kOneOver2Sqrt3);
    auto pair = [&](int c, int d) { return fma(x[c], y[d], x[d] * y[c]); };
    // 0-based: 1 -> 0, ..., 8 -> 7
    {
        T t = pair(3, 5);
        t = fma(x[4], y[6], t);
        t = fma(x[6], y[4], t);
        acc[0] = fma(q, t, fma(r, pair(0, 7), acc[0]));
    }
    {
        T t = pair(4, 5);
        t = fma(-x[3], y[6], t);
        t = fma(-x[6], y[3], t);
        acc[1] = fma(q, t, fma(r, pair(1, 7), acc[1]));
    }
    {
        T t = x[3] * y[3];
        t = fma(x[4], y[4], t);
        t = fma(-x[5], y[5], t);
        t = fma(-x[6], y[6], t);
        acc[2] = fma(q, t, fma(r, pair(2, 7), acc[2]));
    }
    {
        T t = pair(0, 5);
        t = fma(-x[1], y[6], t);
        t = fma(-x[6], y[1], t);
        t = fma(x[2], y[3], t);
        t = fma(x[3], y[2], t);
        acc[3] = fma(q, t, fma(-s, pair(3, 7), acc[3]));
    }
    {
        T t = pair(0, 6);
        t = fma(x[1], y[5], t);
        t = fma(x[5], y[1], t);
        t = fma(x[2], y[4], t);
        t = fma(x[4], y[2], t);
        acc[4] = fma(q, t, fma(-s, pair(4, 7), acc[4]));
    }
    {
        T t = pair(0, 3);
        t = fma(x[1], y[4], t);
        t = fma(x[4], y[1], t);
        t = fma(-x[2], y[5], t);
        t = fma(-x[5], y[2], t);
        acc[5] = fma(q, t, fma(-s, pair(5, 7), acc[5]));
    }
    {
        T t = pair(0, 4);
        t = fma(-x[1], y[3], t);
        t = fma(-x[3], y[1], t);
        t = fma(-x[2], y[6], t);
        t = fma(-x[6], y[2], t);
        acc[6] = fma(q, t, fma(-s, pair(6, 7), acc[6]));
    }
    {
        T a = x[0] * y[0];
        a = fma(x[1], y[1], a);
        a = fma(x[2], y[2], a);
        a = fma(-x[7], y[7], a);
        T b = x[3] * y[3];
        b = fma(x[4], y[4], b);
        b = fma(x[5], y[5], b);
        b = fma(x[6], y[6], b);
        acc[7] = fma(r, a, fma(-s, b, acc[7]));
    }
}

// out^a = Im Tr(T^a a b^dagger) without forming the product: the imaginary parts of the diagonal and the
// six off-diagonal entries of a b^dagger, (a b^dagger)_ij = sum_k a_ik conj(b_jk), in mul_na's order
template <typename T, bool HALF = true>
__device__ __forceinline__ void im_tr_generators_of_product_na(const mat3<T> &a, const mat3<T> &b, T *out) {
    auto entry = [&](int i, int j) {
        T re = a.e[i * 3].re * b.e[j * 3].re;
        T im = -a.e[i * 3].re * b.e[j * 3].im;
        re = fma(a.e[i * 3].im, b.e[j * 3].im, re);
        im = fma(a.e[i * 3].im, b.e[j * 3].re, im);
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            re = fma(a.e[i * 3 + k].re, b.e[j * 3 + k].re, re);
            re = fma(a.e[i * 3 + k].im, b.e[j * 3 + k].im, re);
            im = fma(-a.e[i * 3 + k].re, b.e[j * 3 + k].im, im);
            im = fma(a.e[i * 3 + k].im, b.e[j * 3 + k].re, im);
        }
        return cmk(re, im);
    };
    auto diag_im = [&](int i) {
        T im = -a.e[i * 3].re * b.e[i * 3].im;
        im = fma(a.e[i * 3].im, b.e[i * 3].re, im);
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            im = fma(-a.e[i * 3 + k].re, b.e[i * 3 + k].im, im);
            im = fma(a.e[i * 3 + k].im, b.e[i * 3 + k].re, im);
        }
        return im;
    };
    const cpx<T> m01 = entry(0, 1), m10 = entry(1, 0), m02 = entry(0, 2), m20 = entry(2, 0), m12 = entry(1, 2),
                 m21 = entry(2, 1);
    const T i00 = diag_im(0), i11 = diag_im(1), i22 = diag_im(2);
    im_tr_combine<T, HALF>(m01, m10, m02, m20, m12, m21, i00, i11, i22, out);
}

} // namespace lq
