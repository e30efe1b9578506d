// The FP32 issue roof that the marching kernels are measured against: a chain of fused multiply-adds with no memory
// traffic, enough independent chains per thread and warps per SM to keep every FP32 lane busy, timed with CUDA
// events on the caller's stream (mraygb_measure_fp32_rate, include/mraygb.h).  No counterpart in the reference.

#include <cuda_runtime.h>

#include "internal.h"

namespace mraygb
{

namespace
{

constexpr int kChains = 8;  // independent accumulators per thread
constexpr int kUnroll = 16; // FMAs per chain per loop iteration
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) fma_chain_kernel(float *out, int iters, float a, float b)
{
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        x[c] = 1e-3f * (float)(threadIdx.x + c);
    for (int i = 0; i < iters; ++i)
    {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
        {
#pragma unroll
            for (int c = 0; c < kChains; ++c)
                x[c] = fmaf(x[c], a, b);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s += x[c];
    out[blockIdx.x * kThreads + threadIdx.x] = s; // keeps the chains live
}

} // namespace

cudaError_t measure_fp32_rate(int sm_count, cudaStream_t stream, float *scratch, double *tflops)
{
    const int blocks = sm_count * 4;
    const int iters = 4096;
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess)
        return e;
    if ((e = cudaEventCreate(&e1)) != cudaSuccess)
    {
        cudaEventDestroy(e0);
        return e;
    }
    // one warm-up launch, then the timed one
    fma_chain_kernel<<<blocks, kThreads, 0, stream>>>(scratch, iters, 0.99999994f, 1e-7f);
    cudaEventRecord(e0, stream);
    fma_chain_kernel<<<blocks, kThreads, 0, stream>>>(scratch, iters, 0.99999994f, 1e-7f);
    cudaEventRecord(e1, stream);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess)
    {
        const double flops = 2.0 * kChains * kUnroll * (double)iters * (double)blocks * kThreads;
        *tflops = flops / ((double)ms * 1e-3) / 1e12;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return e;
}

size_t fp32_rate_scratch_floats(int sm_count) { return (size_t)sm_count * 4 * kThreads; }

} // namespace mraygb
