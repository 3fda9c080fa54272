// lq_noalloc.cu -- plaquette sums of a caller-owned device link field, with no allocation.
//
// Some callers cannot let a library allocate device memory: runtimes whose device memory is owned by
// one pool or arena (an embedding framework, a memory-capped MPS client), and loops for which the
// device-wide synchronisation implied by cudaMalloc / cudaFree is not acceptable.  Every other entry
// point of this library keeps its buffers in an lq_state, which allocates.  lq_plaquette_sums_noalloc
// serves those callers: it reads links the caller already holds on the device and writes three sums
// to device memory the caller provides.  Its only scratch (one partial sum per block of 128 sites and
// row) lives in the fixed array below, allocated once when the library is loaded on each device and
// held until the process exits.  The array's device address is looked up once per device and kept,
// so it is not valid across a device reset.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "kernels.cuh"
#include "lqgpu.h"

namespace lq {
void set_last_error(const char *text);
}

namespace {

using lq::Geo;

constexpr uint32_t kBlock = 128;
constexpr uint32_t kMaxSlots = 65536;                // partial sums per row
constexpr uint32_t kMaxSites = kMaxSlots * kBlock;   // 8,388,608 sites (48^4 = 5,308,416 fits)
// 3 rows x 65536 doubles = 1.5 MiB on every device that loads the library
static __device__ __align__(256) double g_plaquette_scratch[3 * kMaxSlots];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_by_device[kMaxDevices] = {};

// The device address of g_plaquette_scratch on the current device.  In host code the array's
// name is only a host-side stand-in, so the address must come from cudaGetSymbolAddress, once
// per device, with that device current.
int scratch_on_current_device(double **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        lq::set_last_error("lq_plaquette_sums_noalloc: cudaGetDevice failed");
        return e == cudaErrorNoDevice ? LQ_ERR_NO_DEVICE : LQ_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        lq::set_last_error("lq_plaquette_sums_noalloc: device index beyond 63");
        return LQ_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_by_device[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_plaquette_scratch);
        if (e != cudaSuccess || !p) {
            (void)cudaGetLastError();
            char buf[256];
            snprintf(buf, sizeof(buf), "lq_plaquette_sums_noalloc: cudaGetSymbolAddress failed (%s)",
                     cudaGetErrorName(e));
            lq::set_last_error(buf);
            return LQ_ERR_CUDA;
        }
        g_scratch_by_device[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_by_device[dev];
    return LQ_OK;
}

// Per site, for mu < nu, the plaquette trace Tr(A B^dag), A = U_mu(x) U_nu(x+mu),
// B = U_nu(x) U_mu(x+nu), read straight from the reference's serde layout
// (double[V*D][3 cols][3 rows][re, im]); one partial per block and row.
template <int D>
__global__ void __launch_bounds__(kBlock) k_plaquette_aos(const double *__restrict__ links, Geo<D> g,
                                                          double *__restrict__ partial) {
    const uint32_t site = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    auto load = [&](uint32_t x, int dir, lq::mat3<double> &m) {
        const double *p = links + ((size_t)x * D + dir) * 18;
#pragma unroll
        for (int col = 0; col < 3; ++col)
#pragma unroll
            for (int row = 0; row < 3; ++row)
                m.e[row * 3 + col] = lq::cmk(p[(col * 3 + row) * 2], p[(col * 3 + row) * 2 + 1]);
    };
    if (site < g.V) {
        uint32_t c[D];
        lq::site_coords(g, site, c);
#pragma unroll
        for (int mu = 0; mu < D; ++mu) {
            const uint32_t xpmu = lq::fwd(g, site, c[mu], mu);
            // U_mu(x), once for every plane (mu, nu)
            lq::mat3<double> umu;
            load(site, mu, umu);
#pragma unroll
            for (int nu = mu + 1; nu < D; ++nu) {
                lq::mat3<double> p, q, A, B;
                load(xpmu, nu, q);
                lq::mul_nn(umu, q, A);
                load(site, nu, p);
                load(lq::fwd(g, site, c[nu], nu), mu, q);
                lq::mul_nn(p, q, B);
                double re = 0.0, im = 0.0;
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    re = fma(A.e[k].re, B.e[k].re, re);
                    re = fma(A.e[k].im, B.e[k].im, re);
                    im = fma(A.e[k].im, B.e[k].re, im);
                    im = fma(-A.e[k].re, B.e[k].im, im);
                }
                v[0] += 1.0 - re / 3.0;
                v[1] += re;
                v[2] += im;
            }
        }
    }
    lq::block_reduce_store<3>(v, partial, blockIdx.x, gridDim.x);
}

template <int D> cudaError_t launch(const double *links, uint32_t V, int L, double *scratch, double *out, cudaStream_t st) {
    const uint32_t blocks = (V + kBlock - 1) / kBlock;
    k_plaquette_aos<D><<<blocks, kBlock, 0, st>>>(links, lq::make_geo<D>(V, (uint32_t)L), scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    lq::k_finalize<3><<<1, 1024, 0, st>>>(scratch, blocks, out);
    return cudaGetLastError();
}

} // namespace

extern "C" int lq_plaquette_sums_noalloc(int dim, int L, const double *d_links, double *d_out, void *stream) {
    if (dim == 0) return LQ_ERR_ZERO_DIMENSION;
    if (L < 2) return LQ_ERR_DIM_TOO_SMALL;
    if (dim < 2 || dim > 4) return LQ_ERR_UNSUPPORTED_DIM;
    if (!d_links || !d_out) return LQ_ERR_INVALID_ARGUMENT;
    uint64_t V = 1;
    for (int i = 0; i < dim; ++i) {
        V *= (uint64_t)L;
        if (V > kMaxSites) {
            char buf[256];
            snprintf(buf, sizeof(buf),
                     "lq_plaquette_sums_noalloc: L^D exceeds the limit of %u sites of its fixed scratch array",
                     kMaxSites);
            lq::set_last_error(buf);
            return LQ_ERR_INVALID_ARGUMENT;
        }
    }
    double *scratch = nullptr;
    const int rc = scratch_on_current_device(&scratch);
    if (rc) return rc;
    // every partial read by the final reduction is written by this call first: nothing in
    // the scratch array has to start at zero
    const cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    switch (dim) {
    case 2: e = launch<2>(d_links, (uint32_t)V, L, scratch, d_out, st); break;
    case 3: e = launch<3>(d_links, (uint32_t)V, L, scratch, d_out, st); break;
    default: e = launch<4>(d_links, (uint32_t)V, L, scratch, d_out, st); break;
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        char buf[256];
        snprintf(buf, sizeof(buf), "lq_plaquette_sums_noalloc: launch failed (%s)", cudaGetErrorName(e));
        lq::set_last_error(buf);
        return LQ_ERR_CUDA;
    }
    return LQ_OK;
}
