// uww_query.cu -- queries against built chunks: per-cell triangle ranges
// (Chunk::tris_around, chunk.rs:315-342), a device index of chunk positions
// (World::get_chunk, world.rs:89-91), and the boids' wall-avoidance ray casts
// (boid.rs:175-244 over util::Tri::new / Tri::intersects, util.rs:12-58),
// batched over many query points on the GPU.
//
// Ray-triangle arithmetic is the reference's f32 sequence with every
// operation separately rounded (cgmath does not fuse), so hit distances
// match a CPU restatement bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#define UWW_TABLE_QUAL __device__
#include "mc_tables.h"
#include "uww_internal.h"

namespace uww {
namespace {

// ---- per-cell first index ------------------------------------------------------
// One CTA per chunk: an exclusive scan of 3 * ntri(case) over the cells in
// stream order, which is the order the build writes each cell's indices.
constexpr int kScanThreads = 256;

__global__ void __launch_bounds__(kScanThreads) cell_first_kernel(const uww_chunk_desc* __restrict__ chunks,
                                                                  uint32_t n, const uint8_t* __restrict__ cases,
                                                                  unsigned long long case_capacity,
                                                                  uint32_t* __restrict__ first, unsigned* errflags)
{
    __shared__ uint8_t ntri[256];
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    for (int i = threadIdx.x; i < 256; i += kScanThreads) ntri[i] = UWW_CASE_NTRI[i];
    __syncthreads();
    for (uint32_t c = blockIdx.x; c < n; c += gridDim.x) {
        const uww_chunk_desc d = chunks[c];
        const unsigned long long NC = (unsigned long long)d.cells * d.cells * d.cells;
        if (d.cells < 1 || d.cells > UWW_MAX_CELLS || (unsigned long long)d.cell_offset + NC > case_capacity) {
            if (threadIdx.x == 0) atomicOr(errflags, (unsigned)UWW_ERRFLAG_RANGE);
            continue;
        }
        const uint8_t* cs = cases + d.cell_offset;
        uint32_t* out = first + d.cell_offset;
        // contiguous runs of cells per thread
        const uint32_t per = (uint32_t)((NC + kScanThreads - 1) / kScanThreads);
        const uint32_t c0 = min((uint32_t)NC, threadIdx.x * per), c1 = min((uint32_t)NC, c0 + per);
        uint32_t mine = 0;
        for (uint32_t i = c0; i < c1; ++i) mine += 3u * ntri[cs[i]];
        // block exclusive scan of the run totals
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t incl = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        uint32_t base = 0;
        for (int w = 0; w < warp; ++w) base += warp_sums[w];
        uint32_t run = base + incl - mine;
        for (uint32_t i = c0; i < c1; ++i) {
            out[i] = run;
            run += 3u * ntri[cs[i]];
        }
        __syncthreads();
    }
}

// ---- chunk position index ---------------------------------------------------------
__device__ __forceinline__ uint32_t pos_hash(int x, int y, int z)
{
    uint32_t h = (uint32_t)x * 0x9E3779B1u ^ (uint32_t)y * 0x85EBCA77u ^ (uint32_t)z * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h;
}

// Open addressing with linear probing; slot = chunk index + 1, 0 = empty.  A
// position given twice keeps one of its chunks.
__global__ void chunk_index_kernel(const uww_chunk_desc* __restrict__ chunks, uint32_t n, uint32_t* table,
                                   uint32_t mask, unsigned* errflags)
{
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const uww_chunk_desc d = chunks[c];
        uint32_t s = pos_hash(d.pos[0], d.pos[1], d.pos[2]) & mask;
        bool placed = false;
        for (uint32_t probe = 0; probe <= mask; ++probe, s = (s + 1) & mask) {
            const uint32_t prev = atomicCAS(&table[s], 0u, c + 1u);
            if (prev == 0u) { placed = true; break; }
            const uww_chunk_desc o = chunks[prev - 1u];
            if (o.pos[0] == d.pos[0] && o.pos[1] == d.pos[1] && o.pos[2] == d.pos[2]) { placed = true; break; }
        }
        if (!placed) atomicOr(errflags, (unsigned)UWW_ERRFLAG_RANGE);
    }
}

__device__ __forceinline__ int chunk_lookup(const uww_ray_scene& sc, int x, int y, int z)
{
    const uint32_t mask = sc.table_size - 1u;
    uint32_t s = pos_hash(x, y, z) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe, s = (s + 1) & mask) {
        const uint32_t v = sc.table[s];
        if (v == 0u) return -1;
        const uww_chunk_desc& d = sc.chunks[v - 1u];
        if (d.pos[0] == x && d.pos[1] == y && d.pos[2] == z) return (int)(v - 1u);
    }
    return -1;
}

// ---- ray casts ------------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ float vdot(V3 a, V3 b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 vcross(V3 a, V3 b)
{
    return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}

constexpr float kRayEpsilon = 1e-5f;  // util.rs:3

// Tri::intersects (util.rs:23-58): the hit distance, or -1.
__device__ __forceinline__ float tri_hit(V3 a, V3 b, V3 c, V3 n, V3 o, V3 d, float range)
{
    const float dn = vdot(n, d);
    if (fabsf(dn) < kRayEpsilon) return -1.f;
    const float t = __fdiv_rn(vdot(n, vsub(a, o)), dn);
    if (t < 0.f || t > range) return -1.f;
    const V3 p = {__fadd_rn(o.x, __fmul_rn(d.x, t)), __fadd_rn(o.y, __fmul_rn(d.y, t)), __fadd_rn(o.z, __fmul_rn(d.z, t))};
    const float d0 = vdot(vcross(vsub(b, a), vsub(p, a)), n);
    const float d1 = vdot(vcross(vsub(c, b), vsub(p, b)), n);
    const float d2 = vdot(vcross(vsub(a, c), vsub(p, c)), n);
    return (d0 >= 0.f && d1 >= 0.f && d2 >= 0.f) ? (t == 0.f ? 0.f : t) : -1.f;
}

constexpr int kQueryWarps = 4;
constexpr int kMaxRays = 32;
constexpr int kTriBuf = 160;  // triangles staged per warp: 32 cells x at most 5

// One warp per query point: the chunks around it (boid.rs:176-207), in each
// the cells within `range` of the point (chunk.rs:315-342).  The warp stages
// the triangles of 32 cells at a time in shared memory (Tri::new's vertices
// and normal, one lane per cell, placed by a warp prefix sum), then tests
// every (triangle, ray) pair with all 32 lanes; the nearest hit per ray is an
// atomic minimum on the float's bits.  The minimum does not depend on the
// order, so the result is the oracle's exactly.
__global__ void __launch_bounds__(kQueryWarps * 32) ray_query_kernel(const uww_ray_scene sc, int chunk_size,
                                                                     const float* __restrict__ origins, uint32_t nq,
                                                                     const float* __restrict__ dirs, uint32_t nrays,
                                                                     int range, float* __restrict__ out)
{
    __shared__ int best[kQueryWarps][kMaxRays];  // bit patterns of non-negative floats order like ints
    __shared__ float rdir[kQueryWarps][kMaxRays * 3];
    __shared__ float4 tri[kQueryWarps][kTriBuf * 3];  // (a, n.x), (b, n.y), (c, n.z)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float cs = (float)chunk_size, rf = (float)range;
    const int R = (int)nrays;
    for (uint32_t q = blockIdx.x * kQueryWarps + warp; q < nq; q += gridDim.x * kQueryWarps) {
        for (int k = lane; k < R; k += 32) best[warp][k] = 0x7f800000;  // +inf
        for (int k = lane; k < 3 * R; k += 32) rdir[warp][k] = dirs[3 * (size_t)q * R + k];
        __syncwarp();
        const V3 o = {origins[3 * (size_t)q], origins[3 * (size_t)q + 1], origins[3 * (size_t)q + 2]};
        int nbuf = 0;  // warp-uniform
        // every (staged triangle, ray) pair, all lanes
        // pair pi = t R + k; lanes step by 32 pairs: t by 32 / R, k by 32 % R
        const int dq = 32 / R, dr = 32 - dq * R;
        auto flush = [&]() {
            const int pairs = nbuf * R;
            int t = lane / R, k = lane - (lane / R) * R;
            for (int pi = lane; pi < pairs; pi += 32) {
                const float4 A = tri[warp][3 * t], B = tri[warp][3 * t + 1], Cc = tri[warp][3 * t + 2];
                const V3 dir = {rdir[warp][3 * k], rdir[warp][3 * k + 1], rdir[warp][3 * k + 2]};
                const float th = tri_hit({A.x, A.y, A.z}, {B.x, B.y, B.z}, {Cc.x, Cc.y, Cc.z}, {A.w, B.w, Cc.w}, o, dir, rf);
                if (th >= 0.f) atomicMin(&best[warp][k], __float_as_int(th));
                t += dq;
                k += dr;
                if (k >= R) {
                    k -= R;
                    ++t;
                }
            }
            __syncwarp();
            nbuf = 0;
        };
        // chunk window, world units (boid.rs:176-182)
        const int sx = (int)floorf(__fdiv_rn(__fsub_rn(o.x, rf), cs)), ex = (int)floorf(__fdiv_rn(__fadd_rn(o.x, rf), cs));
        const int sy = (int)floorf(__fdiv_rn(__fsub_rn(o.y, rf), cs)), ey = (int)floorf(__fdiv_rn(__fadd_rn(o.y, rf), cs));
        const int sz = (int)floorf(__fdiv_rn(__fsub_rn(o.z, rf), cs)), ez = (int)floorf(__fdiv_rn(__fadd_rn(o.z, rf), cs));
        for (int a = sx; a <= ex; ++a)
            for (int b = sy; b <= ey; ++b)
                for (int c = sz; c <= ez; ++c) {
                    const int ci = chunk_lookup(sc, a, b, c);
                    if (ci < 0) continue;
                    const uww_chunk_desc d = sc.chunks[ci];
                    const uww_chunk_record r = sc.records[ci];
                    if (!(r.flags & UWW_CHUNK_HAS_MESH) || (r.flags & UWW_CHUNK_OVERFLOW)) continue;
                    const int N = (int)d.cells;
                    const float nf = (float)N;
                    // tris_around: the cell window around the point's cell
                    const float px = __fdiv_rn(__fsub_rn(o.x, __fmul_rn((float)a, cs)), cs);
                    const float py = __fdiv_rn(__fsub_rn(o.y, __fmul_rn((float)b, cs)), cs);
                    const float pz = __fdiv_rn(__fsub_rn(o.z, __fmul_rn((float)c, cs)), cs);
                    const int mx = (int)floorf(__fmul_rn(px, nf)), my = (int)floorf(__fmul_rn(py, nf)),
                              mz = (int)floorf(__fmul_rn(pz, nf));
                    const int x0 = max(mx - range, 0), y0 = max(my - range, 0), z0 = max(mz - range, 0);
                    const int x1 = min(mx + range, N - 1), y1 = min(my + range, N - 1), z1 = min(mz + range, N - 1);
                    if (x0 > x1 || y0 > y1 || z0 > z1) continue;
                    const int wy = y1 - y0 + 1, wz = z1 - z0 + 1;
                    const int cells = (x1 - x0 + 1) * wy * wz;
                    for (int w0 = 0; w0 < cells; w0 += 32) {
                        const int w = w0 + lane;
                        int nt = 0;
                        uint32_t f = 0;
                        if (w < cells) {
                            const int x = x0 + w / (wy * wz), y = y0 + (w / wz) % wy, z = z0 + w % wz;
                            const uint32_t cell = d.cell_offset + (uint32_t)((x * N + y) * N + z);
                            nt = __ldg(&UWW_CASE_NTRI[sc.cases[cell]]);
                            if (nt) {
                                const uint32_t fl = sc.cell_first[cell];
                                // a scene assembled from different builds is skipped, not read out of range
                                if ((unsigned long long)fl + 3ull * nt > r.num_inds) nt = 0;
                                f = r.ind_offset + fl;
                            }
                        }
                        int incl = nt;
#pragma unroll
                        for (int sh = 1; sh < 32; sh <<= 1) {
                            const int v = __shfl_up_sync(0xffffffffu, incl, sh);
                            if (lane >= sh) incl += v;
                        }
                        const int total = __shfl_sync(0xffffffffu, incl, 31);
                        if (total == 0) continue;
                        if (nbuf + total > kTriBuf) flush();
                        const int base = nbuf + incl - nt;
                        for (int j = 0; j < nt; ++j) {
                            V3 vv[3];
                            bool ok = true;
#pragma unroll
                            for (int m = 0; m < 3; ++m) {
                                const uint32_t id = sc.inds[f + 3 * j + m];
                                ok = ok && id < r.num_verts;
                                const uww_vert_color vc = sc.verts[r.vert_offset + min(id, r.num_verts - 1u)];
                                vv[m] = {vc.pos[0], vc.pos[1], vc.pos[2]};
                            }
                            // Tri::new (util.rs:12-21): normal = safe_normalize((b - a) x (c - a));
                            // a triangle with an index out of range gets a zero normal, which no ray hits
                            V3 nn = {0.f, 0.f, 0.f};
                            if (ok) {
                                nn = vcross(vsub(vv[1], vv[0]), vsub(vv[2], vv[0]));
                                const float mag = __fsqrt_rn(vdot(nn, nn));
                                if (mag != 0.f) nn = {__fdiv_rn(nn.x, mag), __fdiv_rn(nn.y, mag), __fdiv_rn(nn.z, mag)};
                            }
                            float4* T = &tri[warp][3 * (base + j)];
                            T[0] = make_float4(vv[0].x, vv[0].y, vv[0].z, nn.x);
                            T[1] = make_float4(vv[1].x, vv[1].y, vv[1].z, nn.y);
                            T[2] = make_float4(vv[2].x, vv[2].y, vv[2].z, nn.z);
                        }
                        nbuf += total;
                        __syncwarp();
                    }
                }
        if (nbuf) flush();
        for (int k = lane; k < R; k += 32) {
            const int bb = best[warp][k];
            out[(size_t)q * R + k] = bb == 0x7f800000 ? -1.f : __int_as_float(bb);
        }
        __syncwarp();
    }
}

}  // namespace
}  // namespace uww

using namespace uww;

#pragma GCC visibility push(default)
extern "C" {

int uww_cell_tri_offsets(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, const uint8_t* d_cases,
                         uint64_t case_capacity, uint32_t* d_first)
{
    if (!ctx) return UWW_ERR_INVALID_ARG;
    if (n == 0) return UWW_OK;
    if (!d_chunks || !d_cases || !d_first) return UWW_ERR_INVALID_ARG;
    const int grid = (int)std::min<uint32_t>(n, (uint32_t)ctx->num_sms * 8);
    if (!ctx->d_sample_err) {
        cudaError_t e = cudaMalloc((void**)&ctx->d_sample_err, sizeof(unsigned int));
        if (e != cudaSuccess) {
            ctx->d_sample_err = nullptr;
            return status_from_cuda(e, "cudaMalloc");
        }
    }
    cudaError_t e = cudaMemsetAsync(ctx->d_sample_err, 0, sizeof(unsigned int), ctx->stream);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaMemsetAsync");
    cell_first_kernel<<<grid, kScanThreads, 0, ctx->stream>>>(d_chunks, n, d_cases, case_capacity, d_first,
                                                             ctx->d_sample_err);
    return status_from_cuda(cudaGetLastError(), "cell offsets kernel launch");
}

int uww_chunk_index(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t* d_table, uint32_t table_size)
{
    if (!ctx || !d_table) return UWW_ERR_INVALID_ARG;
    if (table_size == 0 || (table_size & (table_size - 1)) || table_size < n) return UWW_ERR_INVALID_ARG;
    if (n && !d_chunks) return UWW_ERR_INVALID_ARG;
    cudaError_t e = cudaMemsetAsync(d_table, 0, (size_t)table_size * sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaMemsetAsync");
    if (n == 0) return UWW_OK;
    if (!ctx->d_sample_err) {
        e = cudaMalloc((void**)&ctx->d_sample_err, sizeof(unsigned int));
        if (e != cudaSuccess) {
            ctx->d_sample_err = nullptr;
            return status_from_cuda(e, "cudaMalloc");
        }
    }
    e = cudaMemsetAsync(ctx->d_sample_err, 0, sizeof(unsigned int), ctx->stream);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaMemsetAsync");
    const int grid = (int)std::min<uint32_t>((n + 255) / 256, (uint32_t)ctx->num_sms * 8);
    chunk_index_kernel<<<grid, 256, 0, ctx->stream>>>(d_chunks, n, d_table, table_size - 1u, ctx->d_sample_err);
    return status_from_cuda(cudaGetLastError(), "chunk index kernel launch");
}

int uww_ray_query(uww_ctx* ctx, const uww_ray_scene* scene, const float* d_origins, uint32_t nq, const float* d_dirs,
                  uint32_t nrays, int32_t range, float* d_t)
{
    if (!ctx || !scene) return UWW_ERR_INVALID_ARG;
    if (nrays == 0 || nrays > (uint32_t)kMaxRays || range < 0) return UWW_ERR_INVALID_ARG;
    if (nq == 0) return UWW_OK;
    if (!d_origins || !d_dirs || !d_t) return UWW_ERR_INVALID_ARG;
    const uww_ray_scene& s = *scene;
    if (!s.chunks || !s.records || !s.verts || !s.inds || !s.cases || !s.cell_first || !s.table) return UWW_ERR_INVALID_ARG;
    if (s.table_size == 0 || (s.table_size & (s.table_size - 1))) return UWW_ERR_INVALID_ARG;
    const int grid = (int)std::min<uint32_t>((nq + kQueryWarps - 1) / kQueryWarps, (uint32_t)ctx->num_sms * 16);
    ray_query_kernel<<<grid, kQueryWarps * 32, 0, ctx->stream>>>(s, ctx->dev.chunk_size, d_origins, nq, d_dirs, nrays,
                                                                 range, d_t);
    return status_from_cuda(cudaGetLastError(), "ray query kernel launch");
}

}  // extern "C"
#pragma GCC visibility pop
