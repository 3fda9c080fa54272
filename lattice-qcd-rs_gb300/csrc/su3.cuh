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

// ---- loads / stores of one link from structure-of-arrays planes ----
// Plane k (k = row*3 + col) of direction mu holds entry k of U_mu for every site:
//   U[(mu*9 + k) * V + site], one complex (double2 / float2) per element.
template <typename T>
__device__ __forceinline__ void load_link(const typename vec2_t<T>::type *__restrict__ U, size_t plane0, size_t V,
                                          uint32_t site, mat3<T> &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const typename vec2_t<T>::type v = __ldg(U + plane0 + (size_t)k * V + site);
        m.e[k] = cmk<T>(v.x, v.y);
    }
}

template <typename T>
__device__ __forceinline__ void store_link(typename vec2_t<T>::type *__restrict__ U, size_t plane0, size_t V,
                                           uint32_t site, const mat3<T> &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        typename vec2_t<T>::type v;
        v.x = m.e[k].re;
        v.y = m.e[k].im;
        U[plane0 + (size_t)k * V + site] = v;
    }
}

} // namespace lq
