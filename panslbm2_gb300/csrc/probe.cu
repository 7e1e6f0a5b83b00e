// probe.cu -- device rate probes for roofline denominators the driver does not measure: the
// FP64 fused multiply-add throughput of the CUDA cores (the FP64 collide kinds are bound by it
// on GB300, whose FP64 rate is a small fraction of its FP32 rate).
#include <cuda_runtime.h>

#include "../../include/panslbm_gb300.h"
#include "launch.h"

namespace {

constexpr int kChains = 8;

// every thread runs kChains independent FMA chains for `iters` iterations; the sum is stored so
// the work is not removed
__global__ void k_fp64_fma(int iters, double a, double b, double *sink) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-9 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.678) sink[blockIdx.x] = s;   // practically never: keeps the chains live
}

}  // namespace

extern "C" int pl_probe_fp64_fma(double *tflops) {
    if (!tflops) return pl::record_error(PL_ERR_ARG, "tflops is NULL");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(double) * 4096) != cudaSuccess) {
        cudaGetLastError();
        return pl::record_error(PL_ERR_ALLOC, "probe buffer");
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    k_fp64_fma<<<blocks, threads>>>(64, 0.999999, 1e-7, sink);   // warm-up
    cudaEventRecord(e0);
    k_fp64_fma<<<blocks, threads>>>(iters, 0.999999, 1e-7, sink);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess || ms <= 0.f) return pl::record_error(PL_ERR_CUDA, "probe kernel failed");
    const double flops = 2.0 * kChains * double(iters) * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return PL_OK;
}
