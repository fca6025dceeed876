// peak.cu — FMA throughput microbenchmarks (the FP32 and FP64 roofline peaks).
//
// Each thread runs kChains independent fused-multiply-add chains so the pipes
// stay full; the grid is a multiple of the SM count. The result is reported as
// FLOP/s with one FMA = 2 FLOPs. The chains' values are written out so the
// compiler cannot drop them.
#include <cuda_runtime.h>

#include "cmg_util.h"

namespace cmg::gpu {

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chain(T* __restrict__ out, int iters, T a, T b) {
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = static_cast<T>(threadIdx.x + c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = x[c] * a + b;  // contracted to one FMA
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
double run(int iters) {
    int dev = 0, sms = 0;
    CMG_CUDA(cudaGetDevice(&dev));
    CMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    CMG_CUDA(cudaMalloc(&out, sizeof(T) * blocks * threads));
    cudaEvent_t e0, e1;
    CMG_CUDA(cudaEventCreate(&e0));
    CMG_CUDA(cudaEventCreate(&e1));
    // a, b keep the chain bounded: x -> x*a + b converges (|a| < 1)
    const T a = static_cast<T>(0.999), b = static_cast<T>(0.001);
    k_fma_chain<T><<<blocks, threads>>>(out, iters / 8, a, b);  // warm-up
    CMG_CUDA(cudaEventRecord(e0));
    k_fma_chain<T><<<blocks, threads>>>(out, iters, a, b);
    CMG_CUDA(cudaEventRecord(e1));
    CMG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    CMG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double fma = static_cast<double>(blocks) * threads * iters * kChains;
    return 2.0 * fma / (ms * 1e-3);
}

}  // namespace

double peak_flops(bool fp64) { return fp64 ? run<double>(1 << 12) : run<float>(1 << 16); }

}  // namespace cmg::gpu
