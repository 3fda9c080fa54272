// su3.cuh -- 3x3 complex matrix arithmetic for the device (CUDA cores, FMA chains).
//
// SU(3) products are 3x3 complex contractions (27 complex multiply-adds): too small and
// too irregular for tensor cores, so they run as FMA chains in registers, templated on
// the storage/compute type T (double or float).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lq {

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

// ---- tiled structure-of-arrays storage ----
// Sites are grouped in tiles of 32 consecutive sites (one warp).  An array of P planes stores
// plane p of site s at ((s / 32) * P + p) * 32 + s % 32: within a tile all planes of a site
// are 32 elements apart, so a thread addresses a whole link with one base pointer and
// constant offsets, and a warp reads each plane of its tile as one contiguous segment.
constexpr int kTile = 32;
__host__ __device__ __forceinline__ size_t tix(uint32_t site, int nplanes, int plane) {
    return ((size_t)(site >> 5) * nplanes + plane) * kTile + (site & 31);
}
__host__ __device__ __forceinline__ uint32_t tiles_of(uint32_t V) { return (V + kTile - 1) / kTile; }

// one link matrix from its 9 complex planes starting at p (entry k at p[k * 32])
template <typename T> __device__ __forceinline__ void load_mat(const typename vec2_t<T>::type *__restrict__ p, mat3<T> &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const typename vec2_t<T>::type v = __ldg(p + k * kTile);
        m.e[k] = cmk<T>(v.x, v.y);
    }
}
template <typename T> __device__ __forceinline__ void store_mat(typename vec2_t<T>::type *__restrict__ p, const mat3<T> &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        typename vec2_t<T>::type v;
        v.x = m.e[k].re;
        v.y = m.e[k].im;
        p[k * kTile] = v;
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
template <typename T> __device__ __forceinline__ void im_tr_generators_of_product(const mat3<T> &a, const mat3<T> &b, T *out) {
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
    const T h = T(0.5);
    out[0] = h * (m10.im + m01.im);
    out[1] = h * (m01.re - m10.re);
    out[2] = h * (i00 - i11);
    out[3] = h * (m20.im + m02.im);
    out[4] = h * (m02.re - m20.re);
    out[5] = h * (m21.im + m12.im);
    out[6] = h * (m12.re - m21.re);
    out[7] = T(kOneOver2Sqrt3) * (i00 + i11) + T(kMinusOneOverSqrt3) * i22;
}

} // namespace lq
