// bench_probe.cu -- measurement kernels for bench.py, built into their own
// library (libuww_bench_probe.so); not part of the chunk builder's ABI.
//
//   * bench_probe_fma: the FP32 peak the noise stage is measured against.
//     Every thread runs 8 independent FMA chains (enough to cover the FMA
//     latency), with no memory traffic but one store per thread at the end
//     that keeps the chains live.
//   * bench_probe_host_write: device-to-host bandwidth of SM stores into
//     page-locked host memory (the streamed host output of the batched
//     build), 16-byte stores by a grid-stride loop.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

__global__ void __launch_bounds__(256) fma_probe_kernel(uint32_t iters, float seed, float* __restrict__ sink)
{
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.9999999f, c = 1e-7f;
    for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    sink[blockIdx.x * blockDim.x + threadIdx.x] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
}

__global__ void host_write_kernel(const uint4* __restrict__ src, uint4* dst, size_t n16)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = src[i];
}

}  // namespace

extern "C" {

// `blocks` CTAs of 256 threads, iters * 128 FMAs per thread; *flops = 2 per FMA.
// d_sink: blocks * 256 floats.  Asynchronous on `stream`; returns a cudaError_t.
int bench_probe_fma(uint32_t blocks, uint32_t iters, float* d_sink, void* stream, double* flops)
{
    if (!d_sink || blocks == 0 || iters == 0) return (int)cudaErrorInvalidValue;
    if (flops) *flops = 2.0 * 8.0 * 16.0 * (double)iters * 256.0 * (double)blocks;
    fma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(iters, 1.0f, d_sink);
    return (int)cudaGetLastError();
}

// Copy `bytes` (a multiple of 16) from device memory into page-locked host
// memory h_dst (cudaHostAlloc / pinned) with `blocks` CTAs of 256 threads
// storing through the device's view of that memory.  Asynchronous.
int bench_probe_host_write(const void* d_src, void* h_dst, size_t bytes, uint32_t blocks, void* stream)
{
    if (!d_src || !h_dst || (bytes & 15) || blocks == 0) return (int)cudaErrorInvalidValue;
    void* dst = nullptr;
    cudaError_t e = cudaHostGetDevicePointer(&dst, h_dst, 0);
    if (e != cudaSuccess) return (int)e;
    host_write_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(static_cast<const uint4*>(d_src),
                                                                static_cast<uint4*>(dst), bytes / 16);
    return (int)cudaGetLastError();
}

}  // extern "C"
