// uww_sample.cu -- density samples of a batch of chunks without the mesher:
// Chunk::build_iso (chunk.rs:105-129) for many chunks, as uww_sample_chunks.
//
// Fast build: one thread per (x, y) sample column, as in the batched build,
// but with the column's samples accumulated in registers: the kernel holds
// nothing else, so it runs at high occupancy and its samples go to global
// memory through a shared-memory staging tile in coalesced rows.  The
// arithmetic is the batched build's (sample_columns_fast) operation for
// operation, so both give the same samples.  Parity build: one thread per
// sample, density<ExactOps> in the reference's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "uww_internal.h"
#include "uww_noise.cuh"

namespace uww {
namespace {

struct SampleArgs {
    const uww_chunk_desc* chunks;
    uint32_t n;
    uint32_t max_cells;
    float* samples;
    unsigned long long capacity;   // floats at samples
    unsigned int* errflags;        // UWW_ERRFLAG_* (device word)
};

// z tables of one chunk for the register columns: per octave and z the
// fraction and its fade, the z lattice cell, and a mask of the z where a new
// cell (run) starts; the depth bias per z.
struct ZRegTable {
    float2 dzc[UWW_MAX_OCTAVES][32];
    int cell[UWW_MAX_OCTAVES][32];
    unsigned mask[UWW_MAX_OCTAVES];
    float bias[32];
};

__device__ void zreg_table(const DevParams& p, ZRegTable& Z, int S, float s, int oz)
{
    const int K = p.octaves, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const float zoff = __fadd_rn((float)oz, p.offset[2]);
    for (int k = warp; k < K; k += nwarps) {
        const bool on = lane < S;
        float dz, fd, dzp, fdp;
        int cell, cellp;
        z_entry(p, k, lane, s, zoff, dz, fd, cell);
        z_entry(p, k, lane - 1, s, zoff, dzp, fdp, cellp);
        const unsigned m = __ballot_sync(0xffffffffu, on && (lane == 0 || cellp != cell));
        if (on) {
            Z.dzc[k][lane] = make_float2(dz, fd);
            Z.cell[k][lane] = cell;
        }
        if (lane == 0) Z.mask[k] = m;
    }
    for (int z = threadIdx.x; z < S; z += blockDim.x) Z.bias[z] = z_bias(p, z, s, oz);
}

// The S samples of every column of one chunk into out[col * S + z]; returns
// nothing (no blank vote here).  Runs are the same for every column, so the
// run-start branches are uniform.
template <int S>
__device__ __forceinline__ void columns_reg(const DevParams& p, const uint8_t* __restrict__ P,
                                            const float4* __restrict__ gp, const ZRegTable& Z, float* out, int ox,
                                            int oy, float s, float norm)
{
    constexpr int SS = S * S;
    const int K = p.octaves;
    const float bf = p.base_freq;
    for (int col = threadIdx.x; col < SS; col += blockDim.x) {
        const int x = col / S, y = col - x * S;
        const float nx = column_coord((float)x, s, ox, p.offset[0], bf);
        const float ny = column_coord((float)y, s, oy, p.offset[1], bf);
        float acc[S];
#pragma unroll
        for (int z = 0; z < S; ++z) acc[z] = Z.bias[z];
        for (int k = 0; k < K; ++k) {
            const ColumnOctave co = column_octave(p, P, nx, ny, k, norm);
            const unsigned mask = Z.mask[k];
            float SA0 = 0.f, SG0 = 0.f, SA1 = 0.f, SG1 = 0.f;
            RunPoly q = {0.f, 0.f, 0.f, 0.f};
            int prev = 0;
#pragma unroll
            for (int z = 0; z < S; ++z) {
                if (mask & (1u << z)) {
                    const int c = Z.cell[k][z];
                    if (z > 0 && c == prev + 1) {
                        SA0 = SA1;
                        SG0 = SG1;
                    } else {
                        column_face(co, gp, c & 255, SA0, SG0);
                    }
                    column_face(co, gp, (c + 1) & 255, SA1, SG1);
                    prev = c;
                    q = run_poly(SA0, SG0, SA1, SG1);
                }
                acc[z] = __fadd_rn(run_value(q, Z.dzc[k][z]), acc[z]);
            }
        }
        float* o = out + col * S;
#pragma unroll
        for (int z = 0; z < S; ++z) o[z] = acc[z];
    }
}

// bytes of the staging tile for MAXS samples per edge; the z tables follow it
// and hold float2/int2 entries, so it is rounded to 16 bytes
__host__ __device__ constexpr size_t stage_bytes(int maxs)
{
    return ((size_t)maxs * maxs * maxs * sizeof(float) + 15) & ~(size_t)15;
}

// MAXS: largest samples per edge staged in shared memory (and the largest
// register column); chunks above it are written by sample_columns_fast
// straight into the output.
template <int MAXS, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) sample_kernel_fast(const DevParams p, const SampleArgs a)
{
    extern __shared__ __align__(16) uint8_t dyn_smem[];
    __shared__ __align__(16) uint8_t P[256];
    __shared__ float4 gp[256];
    __shared__ ZRegTable Z;
    for (int i = threadIdx.x; i < 64; i += blockDim.x)
        reinterpret_cast<uint32_t*>(P)[i] = reinterpret_cast<const uint32_t*>(p.perm)[i];
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        float gx, gy, gz;
        grad_vec(P[i], gx, gy, gz);
        gp[i] = make_float4(gx, gy, gz, 0.f);
    }
    const float norm = fbm_norm(p);
    float* stage = reinterpret_cast<float*>(dyn_smem);
    for (uint32_t c = blockIdx.x; c < a.n; c += gridDim.x) {
        const uww_chunk_desc d = a.chunks[c];
        const int N = (int)d.cells, S = N + 1;
        const unsigned long long S3 = (unsigned long long)S * S * S;
        if (d.cells < 1 || d.cells > a.max_cells || d.cells > UWW_MAX_CELLS ||
            (unsigned long long)d.sample_offset + S3 > a.capacity) {
            if (threadIdx.x == 0) atomicOr(a.errflags, d.cells < 1 || d.cells > a.max_cells ? (unsigned)UWW_ERRFLAG_BAD
                                                                                             : (unsigned)UWW_ERRFLAG_RANGE);
            continue;
        }
        const int ox = d.pos[0] * p.chunk_size, oy = d.pos[1] * p.chunk_size, oz = d.pos[2] * p.chunk_size;
        const float s = __fdiv_rn((float)p.chunk_size, (float)N);
        float* dst = a.samples + d.sample_offset;
        __syncthreads();  // the previous chunk's tables and staging are free
        if (S <= 32 && S <= MAXS && (S == 13 || S == 17 || S == 25)) {
            zreg_table(p, Z, S, s, oz);
            __syncthreads();
            if (S == 13) columns_reg<13>(p, P, gp, Z, stage, ox, oy, s, norm);
            if (MAXS >= 17 && S == 17) columns_reg<(MAXS >= 17 ? 17 : 13)>(p, P, gp, Z, stage, ox, oy, s, norm);
            if (MAXS >= 25 && S == 25) columns_reg<(MAXS >= 25 ? 25 : 13)>(p, P, gp, Z, stage, ox, oy, s, norm);
            __syncthreads();
            for (int i = threadIdx.x; i < (int)S3; i += blockDim.x) dst[i] = stage[i];
        } else {
            // other sizes: the batched build's column noise, in shared memory when
            // the chunk fits the staging tile, else in the output itself
            uint8_t* zt = reinterpret_cast<uint8_t*>(stage) + stage_bytes(MAXS);
            const bool staged = S <= MAXS;
            float* rho = staged ? stage : dst;
            if (staged) sample_columns_fast<false>(p, P, gp, ztable_at(zt, S, p.octaves), rho, N, ox, oy, oz, blockDim.x);
            else sample_columns_fast<true>(p, P, gp, ztable_at(zt, S, p.octaves), rho, N, ox, oy, oz, blockDim.x);
            if (staged) {
                __syncthreads();
                for (int i = threadIdx.x; i < (int)S3; i += blockDim.x) dst[i] = stage[i];
            }
        }
    }
}

__global__ void __launch_bounds__(256) sample_kernel_exact(const DevParams p, const SampleArgs a)
{
    __shared__ __align__(16) uint8_t P[256];
    for (int i = threadIdx.x; i < 64; i += blockDim.x)
        reinterpret_cast<uint32_t*>(P)[i] = reinterpret_cast<const uint32_t*>(p.perm)[i];
    __syncthreads();
    for (uint32_t c = blockIdx.x; c < a.n; c += gridDim.x) {
        const uww_chunk_desc d = a.chunks[c];
        const int N = (int)d.cells, S = N + 1, S2 = S * S;
        const unsigned long long S3 = (unsigned long long)S2 * S;
        if (d.cells < 1 || d.cells > a.max_cells || d.cells > UWW_MAX_CELLS ||
            (unsigned long long)d.sample_offset + S3 > a.capacity) {
            if (threadIdx.x == 0) atomicOr(a.errflags, d.cells < 1 || d.cells > a.max_cells ? (unsigned)UWW_ERRFLAG_BAD
                                                                                             : (unsigned)UWW_ERRFLAG_RANGE);
            continue;
        }
        const float s = __fdiv_rn((float)p.chunk_size, (float)N);
        const int ox = d.pos[0] * p.chunk_size, oy = d.pos[1] * p.chunk_size, oz = d.pos[2] * p.chunk_size;
        for (int idx = threadIdx.x; idx < (int)S3; idx += blockDim.x) {
            const int x = idx / S2, r = idx - x * S2, y = r / S, z = r - y * S;
            const float wx = ExactOps::add(ExactOps::mul((float)x, s), (float)ox);
            const float wy = ExactOps::add(ExactOps::mul((float)y, s), (float)oy);
            const float wz = ExactOps::add(ExactOps::mul((float)z, s), (float)oz);
            a.samples[d.sample_offset + idx] = density<ExactOps, false>(p, P, wx, wy, wz, nullptr);
        }
    }
}

}  // namespace
}  // namespace uww

using namespace uww;

#pragma GCC visibility push(default)
extern "C" {

int uww_sample_chunks(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells, float* d_samples,
                      uint64_t sample_capacity)
{
    if (!ctx) return UWW_ERR_INVALID_ARG;
    if (max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    if (n == 0) return UWW_OK;
    if (!d_chunks || !d_samples) return UWW_ERR_INVALID_ARG;
    cudaStream_t s = ctx->stream;
    if (!ctx->d_sample_err) {
        cudaError_t e = cudaMalloc((void**)&ctx->d_sample_err, sizeof(unsigned int));
        if (e != cudaSuccess) {
            ctx->d_sample_err = nullptr;
            return status_from_cuda(e, "cudaMalloc");
        }
    }
    cudaError_t e = cudaMemsetAsync(ctx->d_sample_err, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaMemsetAsync");
    SampleArgs a;
    std::memset(&a, 0, sizeof(a));
    a.chunks = d_chunks;
    a.n = n;
    a.max_cells = max_cells;
    a.samples = d_samples;
    a.capacity = sample_capacity;
    a.errflags = ctx->d_sample_err;
    const DevParams& p = ctx->dev;
    if (p.math_mode == UWW_MATH_EXACT) {
        const int grid = (int)std::min<uint32_t>(n, (uint32_t)ctx->num_sms * 8);
        sample_kernel_exact<<<grid, 256, 0, s>>>(p, a);
    } else if (max_cells <= 12) {
        const size_t dyn = stage_bytes(13) + ztable_bytes(13, p.octaves);
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sample_kernel_fast<13, 192, 5>, 192, dyn);
        if (e != cudaSuccess) return status_from_cuda(e, "occupancy");
        const int grid = (int)std::min<long long>(n, (long long)std::max(occ, 1) * ctx->num_sms);
        sample_kernel_fast<13, 192, 5><<<grid, 192, dyn, s>>>(p, a);
    } else {
        const size_t dyn = stage_bytes(25) + ztable_bytes((int)max_cells + 1, p.octaves);
        e = cudaFuncSetAttribute(sample_kernel_fast<25, 256, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return status_from_cuda(e, "cudaFuncSetAttribute");
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sample_kernel_fast<25, 256, 2>, 256, dyn);
        if (e != cudaSuccess) return status_from_cuda(e, "occupancy");
        const int grid = (int)std::min<long long>(n, (long long)std::max(occ, 1) * ctx->num_sms);
        sample_kernel_fast<25, 256, 2><<<grid, 256, dyn, s>>>(p, a);
    }
    return status_from_cuda(cudaGetLastError(), "sample kernel launch");
}

int uww_sample_status(uww_ctx* ctx, uint32_t* flags)
{
    if (!ctx || !flags) return UWW_ERR_INVALID_ARG;
    *flags = 0;
    if (!ctx->d_sample_err) return UWW_OK;
    cudaError_t e = cudaMemcpyAsync(flags, ctx->d_sample_err, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return status_from_cuda(e, "uww_sample_status");
}

}  // extern "C"
#pragma GCC visibility pop
