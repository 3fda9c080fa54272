// adjoint.cuh -- reverse-mode adjoint of the symplectic leap-frog (lq_leapfrog_adjoint).
//
// Cotangents: for links, a complex 3x3 matrix lam per link with dO = Re Tr(lam^dag dU)
// (lam = dO/dRe U + i dO/dIm U); for the E-field, 8 reals per link (dO/de^a).  Both are
// stored in the tiled layout of links / E-field (hi arrays only, no compensated part).
//
// Forward step k (the reference's integrate_symplectic fused as in k_md):
//   K_k : E += h_k F(U_k),  F^a = c Im Tr(T^a U Sigma),  c = -sqrt(2/3) / size
//   D_k : U_{k+1} = U_k + kappa i E U_k,  E = sum_a e^a T^a,  kappa = dt sqrt(6) / size
// Reverse step k:
//   adj D_k : lam_E^a += -kappa Im Tr(T^a U_k lam_U^dag);  lam_U <- lam_U - kappa i E lam_U
//   adj K_k : lam_U += h_k c d/dU [sum_l Im Tr(W_l U_l Sigma_l)],  W_l = sum_a lam_E^a(l) T^a
// The last derivative is the vector-Jacobian product of the force: with every plaquette seen
// as a loop U_m X Y Z that starts at link m, W_l enters before a link traversed forward
// (+W_l U_l) and after a link traversed backward (-U_l^dag W_l), and
//   d/dU_m Im Tr(U_m R) = i R^dag,  R = X Y Z W_m + (single W insertions into X Y Z).
#pragma once
#include "kernels.cuh"

namespace lq {

template <typename T> __device__ __forceinline__ void mat_adj(const mat3<T> &a, mat3<T> &r) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.e[i * 3 + j] = cmk(a.e[j * 3 + i].re, -a.e[j * 3 + i].im);
}
template <typename T> __device__ __forceinline__ void mat_axpy(T s, const mat3<T> &x, mat3<T> &y) {
#pragma unroll
    for (int k = 0; k < 9; ++k) y.e[k] = cmk(fma(s, x.e[k].re, y.e[k].re), fma(s, x.e[k].im, y.e[k].im));
}

// lam_U(m) = scale * Sigma_m^dag: the cotangent of scale * sum_P Re Tr P at the links U
template <int D, typename T>
__global__ void __launch_bounds__(128) k_adj_init(const V2<T> *__restrict__ U, V2<T> *__restrict__ lamU, Geo<D> g,
                                                  T scale) {
    const uint32_t site = (blockIdx.x / D) * blockDim.x + threadIdx.x;
    const int mu = blockIdx.x % D;
    if (site >= g.V) return;
    uint32_t c[D];
    site_coords(g, site, c);
    mat3<T> sig, r;
    staple_sum<D, T>(U, g, site, c, mu, sig);
    mat_adj(sig, r);
#pragma unroll
    for (int k = 0; k < 9; ++k) r.e[k] = cmk(scale * r.e[k].re, scale * r.e[k].im);
    store_link<T>(lamU, tix(site, D * 9, mu * 9), r);
}

// r += (NEG ? -1 : 1) p W for W = sum_a c^a T^a (Hermitian traceless: real diagonal, lower
// off-diagonal entries the conjugates of the upper ones), multiplied from the right
template <typename T, bool NEG>
__device__ __forceinline__ void mul_adj_acc(const mat3<T> &p, const T *c, mat3<T> &r) {
    const T h = T(0.5);
    const T c8p = T(kOneOver2Sqrt3) * c[7];
    const T d[3] = {h * c[2] + c8p, -h * c[2] + c8p, T(kMinusOneOverSqrt3) * c[7]};
    const cpx<T> e01 = cmk(h * c[0], -h * c[1]), e02 = cmk(h * c[3], -h * c[4]), e12 = cmk(h * c[5], -h * c[6]);
    // W by columns: W_kj for k = 0, 1, 2
    const cpx<T> w[3][3] = {{cmk(d[0], T(0)), cmk(e01.re, -e01.im), cmk(e02.re, -e02.im)},
                            {e01, cmk(d[1], T(0)), cmk(e12.re, -e12.im)},
                            {e02, e12, cmk(d[2], T(0))}};
    const T sg = NEG ? T(-1) : T(1);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T re = r.e[i * 3 + j].re, im = r.e[i * 3 + j].im;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const cpx<T> a = p.e[i * 3 + k], b = w[j][k];
                re = fma(sg * a.re, b.re, re);
                im = fma(sg * a.re, b.im, im);
                if (k != j) { // the diagonal of W is real
                    re = fma(-sg * a.im, b.im, re);
                }
                im = fma(sg * a.im, b.re, im);
            }
            r.e[i * 3 + j] = cmk(re, im);
        }
}

// one plaquette loop U_m X Y Z of link m: R of the loop (see the header comment).  Each of X,
// Y, Z is link `l` traversed forward (fwd = true: U_l) or backward (U_l^dag); cl: lam_E of l.
template <typename T>
__device__ __forceinline__ void loop_r(const mat3<T> (&u)[3], const T (&cl)[3][8], const bool (&fwd)[3],
                                       const mat3<T> &wm, mat3<T> &racc) {
    mat3<T> p, q, t;
    // the first factor
    if (fwd[0]) {
        p = u[0];
        adj_mul<T>(cl[0], u[0], q); // W U
    } else {
        mat_adj(u[0], p);
        adj_mul<T>(cl[0], u[0], t);
        mat_adj(t, q); // (W U)^dag = U^dag W, with the minus sign below
#pragma unroll
        for (int k = 0; k < 9; ++k) q.e[k] = cmk(-q.e[k].re, -q.e[k].im);
    }
    // the product and its single-insertion sum through the next factors as a pair (p, q):
    //   forward U:   (p U, q U + p W U) = (p U, (q + p W) U)
    //   backward U^dag, inserted as -U^dag W:   (p U^dag, q U^dag - (p U^dag) W)
    // one product fewer per factor than forming W U and p (W U) apart
#pragma unroll
    for (int f = 1; f < 3; ++f) {
        mat3<T> np, nq;
        if (fwd[f]) {
            mul_nn(p, u[f], np);
            mul_adj_acc<T, false>(p, cl[f], q); // q + p W
            mul_nn(q, u[f], nq);
        } else {
            mul_na(p, u[f], np);
            mul_na(q, u[f], nq);
            mul_adj_acc<T, true>(np, cl[f], nq);
        }
        p = np;
        q = nq;
    }
    // R = q + p W_m
    mul_nn(p, wm, t);
#pragma unroll
    for (int k = 0; k < 9; ++k)
        racc.e[k] = cmk(racc.e[k].re + q.e[k].re + t.e[k].re, racc.e[k].im + q.e[k].im + t.e[k].im);
}

template <int D, typename T>
__device__ __forceinline__ void load_coef(const T *__restrict__ lamE, uint32_t site, int dir, T (&c)[8]) {
    load_efield<T>(lamE, tix(site, D * 8, dir * 8), c);
}

// lam_U(m) += coef * i * (sum over the 2(D-1) plaquette loops of m of R)^dag, coef = h c
template <int D, typename T>
__global__ void __launch_bounds__(128) k_adj_kick(const V2<T> *__restrict__ U, const T *__restrict__ lamE,
                                                  V2<T> *__restrict__ lamU, Geo<D> g, T coef) {
    const uint32_t site = (blockIdx.x / D) * blockDim.x + threadIdx.x;
    const int mu = blockIdx.x % D;
    if (site >= g.V) return;
    uint32_t c[D];
    site_coords(g, site, c);
    const uint32_t xpmu = fwd(g, site, c[mu], mu);
    mat3<T> wm, racc;
    {
        T cm[8];
        load_coef<D, T>(lamE, site, mu, cm);
        adjoint_to_matrix<T>(cm, wm);
    }
    mat_zero(racc);
#pragma unroll 1
    for (int nu = 0; nu < D; ++nu) {
        if (nu == mu) continue;
        mat3<T> u[3];
        T cl[3][8];
        {
            // upper loop: U_mu(x) U_nu(x+mu) U_mu(x+nu)^dag U_nu(x)^dag
            const uint32_t xpnu = fwd(g, site, c[nu], nu);
            load_link<T>(U, tix(xpmu, D * 9, nu * 9), u[0]);
            load_link<T>(U, tix(xpnu, D * 9, mu * 9), u[1]);
            load_link<T>(U, tix(site, D * 9, nu * 9), u[2]);
            load_coef<D, T>(lamE, xpmu, nu, cl[0]);
            load_coef<D, T>(lamE, xpnu, mu, cl[1]);
            load_coef<D, T>(lamE, site, nu, cl[2]);
            const bool f[3] = {true, false, false};
            loop_r<T>(u, cl, f, wm, racc);
        }
        {
            // lower loop: U_mu(x) U_nu(x+mu-nu)^dag U_mu(x-nu)^dag U_nu(x-nu)
            const uint32_t xmnu = bwd(g, site, c[nu], nu);
            const uint32_t xpmu_mnu = bwd(g, xpmu, c[nu], nu);
            load_link<T>(U, tix(xpmu_mnu, D * 9, nu * 9), u[0]);
            load_link<T>(U, tix(xmnu, D * 9, mu * 9), u[1]);
            load_link<T>(U, tix(xmnu, D * 9, nu * 9), u[2]);
            load_coef<D, T>(lamE, xpmu_mnu, nu, cl[0]);
            load_coef<D, T>(lamE, xmnu, mu, cl[1]);
            load_coef<D, T>(lamE, xmnu, nu, cl[2]);
            const bool f[3] = {false, false, true};
            loop_r<T>(u, cl, f, wm, racc);
        }
    }
    // += coef * i * racc^dag: i (a - ib) = b + ia for each entry a + ib of racc^T
    const size_t ui = tix(site, D * 9, mu * 9);
    mat3<T> l;
    load_link<T>(lamU, ui, l);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const cpx<T> r = racc.e[j * 3 + i];
            l.e[i * 3 + j].re = fma(coef, r.im, l.e[i * 3 + j].re);
            l.e[i * 3 + j].im = fma(coef, r.re, l.e[i * 3 + j].im);
        }
    store_link<T>(lamU, ui, l);
}

// adjoint of the drift U' = U + kappa i E U at the links U (before the drift) and momenta E:
//   lam_E^a += -kappa Im Tr(T^a U lam_U^dag),  lam_U <- lam_U - kappa i E lam_U
template <int D, typename T>
__global__ void __launch_bounds__(128) k_adj_drift(const V2<T> *__restrict__ U, const T *__restrict__ E,
                                                   V2<T> *__restrict__ lamU, T *__restrict__ lamE, uint32_t V,
                                                   T kappa) {
    const uint32_t site = (blockIdx.x / D) * blockDim.x + threadIdx.x;
    const int mu = blockIdx.x % D;
    if (site >= V) return;
    const size_t ui = tix(site, D * 9, mu * 9), ei = tix(site, D * 8, mu * 8);
    mat3<T> u, lu, lua, x;
    load_link<T>(U, ui, u);
    load_link<T>(lamU, ui, lu);
    mat_adj(lu, lua);
    T f[8], e[8], le[8];
    im_tr_generators_of_product(u, lua, f);
    load_efield<T>(lamE, ei, le);
    load_efield<T>(E, ei, e);
#pragma unroll
    for (int a = 0; a < 8; ++a) le[a] = fma(-kappa, f[a], le[a]);
    store_efield<T>(lamE, ei, le);
    adj_mul<T>(e, lu, x); // E lam_U
    // -kappa i x: -i (a + ib) = b - ia
#pragma unroll
    for (int k = 0; k < 9; ++k) lu.e[k] = cmk(fma(kappa, x.e[k].im, lu.e[k].re), fma(-kappa, x.e[k].re, lu.e[k].im));
    store_link<T>(lamU, ui, lu);
}

// partials of sum_i a_i b_i (hi arrays of n reals)
template <typename T>
__global__ void __launch_bounds__(256) k_dot(const T *__restrict__ a, const T *__restrict__ b, size_t n,
                                             double *__restrict__ partial) {
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        acc = fma((double)a[i], (double)b[i], acc);
    double v[1] = {acc};
    block_reduce_store<1>(v, partial, blockIdx.x, gridDim.x);
}

} // namespace lq
