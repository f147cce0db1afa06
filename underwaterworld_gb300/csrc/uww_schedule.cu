// uww_schedule.cu -- the chunk scheduler's feed on the GPU: World::update_nearby
// (world.rs:148-234) with GenPrio's ordering (world.rs:33-58) and
// util::in_frustum (util.rs:77-85).  Every chunk position around the sub is
// classified against the view and generation frusta; known chunks go to the
// render list, unknown ones to the generation list, sorted so that the
// batched build's work queue (which takes descriptors in order) finishes
// in-view chunks first.  f32 with the reference's operation order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "uww_internal.h"

namespace uww {
namespace {

constexpr int kSchedThreads = 1024;
constexpr int kSchedMax = 4096;  // candidates sorted in shared memory (32 KB of keys)

__device__ __forceinline__ uint32_t pos_hash_s(int x, int y, int z)
{
    uint32_t h = (uint32_t)x * 0x9E3779B1u ^ (uint32_t)y * 0x85EBCA77u ^ (uint32_t)z * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h;
}

// the uww_chunk_index table of the known chunks
__device__ int known_lookup(const uww_chunk_desc* chunks, const uint32_t* table, uint32_t size, int x, int y, int z)
{
    if (!table || size == 0) return -1;
    const uint32_t mask = size - 1u;
    uint32_t s = pos_hash_s(x, y, z) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe, s = (s + 1) & mask) {
        const uint32_t v = table[s];
        if (v == 0u) return -1;
        const uww_chunk_desc& d = chunks[v - 1u];
        if (d.pos[0] == x && d.pos[1] == y && d.pos[2] == z) return (int)(v - 1u);
    }
    return -1;
}

// util::in_frustum: clip = M * (p, 1) for a column-major M, then the
// perspective divide and the wgpu clip volume
__device__ __forceinline__ bool in_frustum(const float* m, float x, float y, float z)
{
    float c[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        c[i] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[i], x), __fmul_rn(m[4 + i], y)), __fmul_rn(m[8 + i], z)),
                         m[12 + i]);
    const float w = c[3];
    const float cx = __fdiv_rn(c[0], w), cy = __fdiv_rn(c[1], w), cz = __fdiv_rn(c[2], w);
    return fabsf(cx) <= 1.f && fabsf(cy) <= 1.f && cz >= 0.f && cz <= 1.f;
}

// float -> u32 with the same order
__device__ __forceinline__ uint32_t float_key(float f)
{
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

struct SchedArgs {
    uww_schedule_params sp;
    int chunk_size;
    const uww_chunk_desc* known;
    const uww_chunk_record* known_records;
    const uint32_t* table;
    uint32_t table_size;
    uww_chunk_desc* generate;
    uint32_t generate_capacity;
    int32_t* render;
    uint32_t render_capacity;
    uint32_t* counts;   // [0] generation list, [1] render list (true lengths, even beyond capacity)
};

// One CTA: classify every candidate, bitonic-sort the generation keys in
// shared memory, write both lists.
__global__ void __launch_bounds__(kSchedThreads) schedule_kernel(const SchedArgs a)
{
    __shared__ unsigned long long keys[kSchedMax];
    __shared__ uint32_t render_flags[kSchedMax / 32];
    __shared__ uint32_t n_gen;
    const uww_schedule_params& sp = a.sp;
    const int G = sp.generation_dist;
    const int sz = max(sp.sub_chunk[2] - G, sp.min_z), ez = min(sp.sub_chunk[2] + G, sp.max_z);
    const int nz = max(ez - sz + 1, 0);
    const int total = 2 * G * 2 * G * nz;
    const float cs = (float)a.chunk_size;
    const float max_view = __fmul_rn((float)sp.view_dist, cs), max_gen = __fmul_rn((float)G, cs);
    if (threadIdx.x == 0) n_gen = 0;
    for (int i = threadIdx.x; i < kSchedMax / 32; i += blockDim.x) render_flags[i] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        // loop order of update_nearby: x, then y, then z
        const int xi = i / (2 * G * nz), yi = (i / nz) % (2 * G), zi = i % nz;
        const int cx = sp.sub_chunk[0] - G + xi, cy = sp.sub_chunk[1] - G + yi, cz = sz + zi;
        const float mx = __fmul_rn(__fadd_rn((float)cx, 0.5f), cs), my = __fmul_rn(__fadd_rn((float)cy, 0.5f), cs),
                    mz = __fmul_rn(__fadd_rn((float)cz, 0.5f), cs);
        const float dx = __fsub_rn(sp.sub_pos[0], mx), dy = __fsub_rn(sp.sub_pos[1], my), dz = __fsub_rn(sp.sub_pos[2], mz);
        const float dist = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        if (dist > max_gen) continue;
        bool in_view = false, in_gen = false;
        // corners in the order of world.rs:171-180
        for (int k = 0; k < 8; ++k) {
            const float ox = (float)(k & 1), oy = (float)((k >> 1) & 1), oz = (float)((k >> 2) & 1);
            const float px = __fmul_rn(__fadd_rn((float)cx, ox), cs), py = __fmul_rn(__fadd_rn((float)cy, oy), cs),
                        pz = __fmul_rn(__fadd_rn((float)cz, oz), cs);
            if (in_frustum(sp.gen_proj, px, py, pz)) {
                in_gen = true;
                if (in_frustum(sp.view_proj, px, py, pz)) {
                    in_view = true;
                    break;
                }
            }
        }
        const int known = known_lookup(a.known, a.table, a.table_size, cx, cy, cz);
        if (known >= 0) {
            const bool not_blank = (a.known_records[known].flags & UWW_CHUNK_HAS_MESH) != 0;
            if (dist < max_view && not_blank && in_view) atomicOr(&render_flags[i >> 5], 1u << (i & 31));
        } else {
            // GenPrio::compare: in view, then in the generation frustum, then dist^2 + z
            const float prio = __fadd_rn(__fmul_rn(dist, dist), __fmul_rn((float)cz, cs));
            const unsigned long long cls = in_view ? 0ull : in_gen ? 1ull : 2ull;
            const uint32_t slot = atomicAdd(&n_gen, 1u);
            keys[slot] = (cls << 62) | ((unsigned long long)float_key(prio) << 30) | (unsigned long long)i;
        }
    }
    __syncthreads();
    const uint32_t ng = n_gen;
    // pad to a power of two and bitonic-sort ascending
    uint32_t np2 = 1;
    while (np2 < ng) np2 <<= 1;
    for (uint32_t i = ng + threadIdx.x; i < np2; i += blockDim.x) keys[i] = ~0ull;
    __syncthreads();
    for (uint32_t k = 2; k <= np2; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < np2; i += blockDim.x) {
                const uint32_t l = i ^ j;
                if (l > i) {
                    const unsigned long long a0 = keys[i], a1 = keys[l];
                    const bool up = (i & k) == 0;
                    if ((a0 > a1) == up) { keys[i] = a1; keys[l] = a0; }
                }
            }
            __syncthreads();
        }
    // generation list in processing order, laid out like uww_layout_cells
    const uint32_t cells = sp.cells, nc = cells * cells * cells, ns = (cells + 1) * (cells + 1) * (cells + 1);
    for (uint32_t r = threadIdx.x; r < ng && r < a.generate_capacity; r += blockDim.x) {
        const int i = (int)(keys[r] & 0x3fffffffull);
        const int xi = i / (2 * G * nz), yi = (i / nz) % (2 * G), zi = i % nz;
        uww_chunk_desc d;
        d.pos[0] = sp.sub_chunk[0] - G + xi;
        d.pos[1] = sp.sub_chunk[1] - G + yi;
        d.pos[2] = sz + zi;
        d.cells = cells;
        d.cell_offset = r * nc;
        d.sample_offset = r * ns;
        d.reserved[0] = d.reserved[1] = 0;
        a.generate[r] = d;
    }
    // render list in loop order
    if (threadIdx.x == 0) {
        uint32_t nr = 0;
        for (int w = 0; w < (total + 31) / 32; ++w) {
            uint32_t bits = render_flags[w];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1;
                const int i = w * 32 + b;
                if (nr < a.render_capacity) {
                    const int xi = i / (2 * G * nz), yi = (i / nz) % (2 * G), zi = i % nz;
                    a.render[3 * nr] = sp.sub_chunk[0] - G + xi;
                    a.render[3 * nr + 1] = sp.sub_chunk[1] - G + yi;
                    a.render[3 * nr + 2] = sz + zi;
                }
                ++nr;
            }
        }
        a.counts[0] = ng;
        a.counts[1] = nr;
    }
}

}  // namespace
}  // namespace uww

using namespace uww;

#pragma GCC visibility push(default)
extern "C" {

int uww_schedule_chunks(uww_ctx* ctx, const uww_schedule_params* sp, const uww_chunk_desc* d_known,
                        const uww_chunk_record* d_known_records, const uint32_t* d_known_table,
                        uint32_t known_table_size, uww_chunk_desc* d_generate, uint32_t generate_capacity,
                        int32_t* d_render, uint32_t render_capacity, uint32_t* d_counts)
{
    if (!ctx || !sp || !d_generate || !d_render || !d_counts) return UWW_ERR_INVALID_ARG;
    if (sp->generation_dist < 0 || sp->view_dist < 0 || sp->cells < 1 || sp->cells > UWW_MAX_CELLS)
        return UWW_ERR_INVALID_ARG;
    const long long nz = std::max(0, std::min(sp->sub_chunk[2] + sp->generation_dist, sp->max_z) -
                                         std::max(sp->sub_chunk[2] - sp->generation_dist, sp->min_z) + 1);
    const long long total = 4ll * sp->generation_dist * sp->generation_dist * nz;
    if (total > kSchedMax) return UWW_ERR_INVALID_ARG;
    if (d_known_table && (known_table_size == 0 || (known_table_size & (known_table_size - 1)) || !d_known ||
                          !d_known_records))
        return UWW_ERR_INVALID_ARG;
    SchedArgs a;
    std::memset(&a, 0, sizeof(a));
    a.sp = *sp;
    a.chunk_size = ctx->dev.chunk_size;
    a.known = d_known;
    a.known_records = d_known_records;
    a.table = d_known_table;
    a.table_size = d_known_table ? known_table_size : 0;
    a.generate = d_generate;
    a.generate_capacity = generate_capacity;
    a.render = d_render;
    a.render_capacity = render_capacity;
    a.counts = d_counts;
    schedule_kernel<<<1, kSchedThreads, 0, ctx->stream>>>(a);
    return status_from_cuda(cudaGetLastError(), "schedule kernel launch");
}

}  // extern "C"
#pragma GCC visibility pop
