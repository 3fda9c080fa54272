// lq_peak.cu -- arithmetic peak of this GPU for the compute roofline of the FP64 form.
//
// The FP64 form's kernels are bound by the FP64 pipe, not by HBM, on GB300 (its FP64 rate is a small
// fraction of its FP32 rate).  Their roofline fraction needs a measured denominator: this kernel
// runs long chains of independent multiply-adds (8 per thread, no memory traffic) on every SM and
// reports the achieved FLOP/s (2 per multiply-add) from CUDA events, at the clocks the GPU runs at.
#include <cuda_runtime.h>

#include <cstdio>

#include "lqgpu.h"

namespace lq {
void set_last_error(const char *text);
}

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;
constexpr int kThreads = 256;

template <typename T> __global__ void __launch_bounds__(kThreads) k_fma_chains(T b, T c, T *sink, int flag) {
    T a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = T(threadIdx.x + i);
#pragma unroll 16
    for (int it = 0; it < kIters; ++it)
#pragma unroll
        for (int i = 0; i < kChains; ++i) a[i] = fma(a[i], b, c);
    T s = T(0);
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += a[i];
    // never true for the arguments passed: keeps the chains live without memory traffic
    if (flag && s == T(-1)) sink[blockIdx.x] = s;
}

template <typename T> int run(int blocks, double *flops_per_s) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best = 0.0f;
    // b slightly below 1 and c small keep every chain finite and normal for all iterations
    const T b = T(0.99999), c = T(1e-3);
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(e0, 0);
        if (e == cudaSuccess) k_fma_chains<T><<<blocks, kThreads>>>(b, c, (T *)nullptr, 0);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms; // rep 0 warms up
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess || best <= 0.0f) {
        (void)cudaGetLastError();
        char buf[256];
        snprintf(buf, sizeof(buf), "lq_fma_peak: %s", cudaGetErrorName(e));
        lq::set_last_error(buf);
        return e == cudaErrorNoDevice ? LQ_ERR_NO_DEVICE : LQ_ERR_CUDA;
    }
    const double flops = 2.0 * kChains * (double)kIters * (double)blocks * kThreads;
    *flops_per_s = flops / (best * 1e-3);
    return LQ_OK;
}

} // namespace

extern "C" int lq_fma_peak(int precision, double *flops_per_s) {
    if (!flops_per_s) return LQ_ERR_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        lq::set_last_error("lq_fma_peak: no CUDA device");
        return LQ_ERR_NO_DEVICE;
    }
    // 8 resident blocks of 256 threads per SM: full occupancy of the multiply-add pipes
    const int blocks = sms * 8;
    if (precision == LQ_PRECISION_F64) return run<double>(blocks, flops_per_s);
    if (precision == LQ_PRECISION_F32) return run<float>(blocks, flops_per_s);
    return LQ_ERR_INVALID_ARGUMENT;
}
