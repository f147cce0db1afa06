// uww_build.cu -- the chunk-build kernel (noise + marching cubes + emission).
//
// One CTA builds one chunk at a time:
//   1. samples the (N+1)^3 density grid (Chunk::build_iso, chunk.rs:105-129)
//      into shared memory, and votes the early blank check (chunk.rs:131-133);
//   2. classifies every cell to its 8-bit case (chunk.rs:144-162), counts its
//      triangles and the vertices it creates, and block-scans those counts in
//      the reference's cell order (x outer, y, z inner; chunk.rs:138-142);
//   3. (batched form) takes the chunk's output offsets from a decoupled
//      look-back over the work-queue order, so the batch is laid out compact
//      and in chunk order in one pass;
//   4. walks the active cells' triangle rows (chunk.rs:164-251) and writes
//      chunk-local u32 indices and, once per vertex, VertColor + normal.
//
// Vertex dedup (chunk.rs:233) is resolved without a search: a crossed edge is
// referenced by every cell that holds it, so the vertex the reference creates
// for it is made by the first such cell in stream order (its "owner"), at the
// owner's first reference to that edge.  Vertex ids are the running count of
// owned first references, scanned over cells.
//
// The batched form runs as a persistent grid fed by an atomic ticket
// counter; the plain form (one chunk per launch) is the same code without the
// queue and look-back.
#include <cuda_runtime.h>

#define UWW_TABLE_QUAL __constant__
#include "mc_tables.h"
#include "uww_internal.h"

namespace uww {

namespace {

struct SmemTables {
    int8_t tri[256][16];
    uint16_t edges[256];
    uint8_t ntri[256];
    uint8_t perm[256];
    int8_t share[12][4][5];
    uint8_t corners[12][2];
    uint16_t owned[2][64];        // [oriented?][boundary flags] -> owned edge mask
    unsigned long long warp_sums[32];
    unsigned long long chunk_total;
    unsigned long long excl;       // packed exclusive prefix (verts | inds << 32)
    uint32_t ticket;
    uint32_t fits;
    uint32_t any_inside;
};

__device__ __forceinline__ int boundary_flags(int x, int y, int z, int N)
{
    return (x == 0) | ((y == 0) << 1) | ((z == 0) << 2) | ((x == N - 1) << 3) | ((y == N - 1) << 4) |
           ((z == N - 1) << 5);
}

// First cell (in stream order) holding edge e of cell (x,y,z) -- with the same
// orientation when `oriented` -- and that cell's local edge id.
__device__ __forceinline__ int find_owner(const SmemTables& T, int e, int x, int y, int z, int N, bool oriented,
                                          int& ox, int& oy, int& oz)
{
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int8_t* s = T.share[e][c];
        if (oriented && !s[4]) continue;
        const int cx = x + s[0], cy = y + s[1], cz = z + s[2];
        if (cx < 0 || cy < 0 || cz < 0 || cx >= N || cy >= N || cz >= N) continue;
        ox = cx; oy = cy; oz = cz;
        return s[3];
    }
    ox = x; oy = y; oz = z;  // unreachable: the cell itself is always a candidate
    return e;
}

// Number of distinct owned edges first referenced in `row` before edge e.
__device__ __forceinline__ int rank_in_row(const int8_t* row, unsigned owned, int e)
{
    unsigned seen = 0;
    int r = 0;
    for (int j = 0; j < 16; ++j) {
        const int ej = row[j];
        if (ej < 0 || ej == e) break;
        const unsigned bit = 1u << ej;
        if ((owned & bit) && !(seen & bit)) { seen |= bit; ++r; }
    }
    return r;
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Packed per-cell counts for the block scan: verts [21:0], inds [43:22], active [62:44].
constexpr int kIndShift = 22;
constexpr int kActShift = 44;
constexpr unsigned long long kField22 = (1ull << 22) - 1;

__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v, SmemTables& T,
                                                                   unsigned long long& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    unsigned long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) T.warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < nwarps ? T.warp_sums[lane] : 0ull;
        unsigned long long wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nwarps) T.warp_sums[lane] = wi - w;  // exclusive warp offsets
        if (lane == nwarps - 1) T.chunk_total = wi;
    }
    __syncthreads();
    total = T.chunk_total;
    return T.warp_sums[warp] + incl - v;
}

__device__ __forceinline__ unsigned long long sat_add_packed(unsigned long long a, unsigned long long b)
{
    unsigned long long v = (a & kLbVertMax) + (b & kLbVertMax);
    unsigned long long i = ((a >> 30) & kLbIndMax) + ((b >> 30) & kLbIndMax);
    if (v > kLbVertMax) v = kLbVertMax;
    if (i > kLbIndMax) i = kLbIndMax;
    return v | (i << 30);
}

// Decoupled look-back by warp 0: publishes this ticket's aggregate, sums the
// predecessors' values back to the nearest inclusive prefix, publishes the
// inclusive prefix.  Returns the packed exclusive prefix.  Every wait is
// bounded by spin_limit_cycles; on timeout the prefix saturates (so nothing is
// written out of place) and the error flag is raised.
__device__ unsigned long long lookback(const BuildArgs& a, uint32_t ticket, unsigned long long own)
{
    const int lane = threadIdx.x & 31;
    if (ticket == 0) {
        if (lane == 0) st_release(&a.lookback[0], kLbInclusive | own);
        return 0ull;
    }
    if (lane == 0) st_release(&a.lookback[ticket], kLbAggregate | own);
    unsigned long long sum = 0ull;
    long long j = (long long)ticket - 1;
    const long long t0 = clock64();
    bool timed_out = false;
    for (;;) {
        const long long idx = j - lane;
        const unsigned long long s = idx >= 0 ? ld_acquire(&a.lookback[idx]) : kLbInclusive;
        const unsigned status = (unsigned)(s >> 62);
        if (__any_sync(0xffffffffu, status == 0)) {
            if (clock64() - t0 > a.spin_limit_cycles) { timed_out = true; break; }
            __nanosleep(64);
            continue;
        }
        const unsigned incl = __ballot_sync(0xffffffffu, status == 2);
        const int first = incl ? __ffs(incl) - 1 : 31;
        unsigned long long mine = lane <= first ? (s & ~(3ull << 62)) : 0ull;
        unsigned long long v = mine & kLbVertMax, i = (mine >> 30) & kLbIndMax;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v += __shfl_xor_sync(0xffffffffu, v, o);
            i += __shfl_xor_sync(0xffffffffu, i, o);
        }
        sum = sat_add_packed(sum, (v > kLbVertMax ? kLbVertMax : v) | ((i > kLbIndMax ? kLbIndMax : i) << 30));
        if (incl) break;
        j -= 32;
    }
    if (timed_out) {
        sum = kLbVertMax | (kLbIndMax << 30);
        if (lane == 0) atomicOr(&a.totals[3], kErrTimeout);
    }
    if (lane == 0) st_release(&a.lookback[ticket], kLbInclusive | sat_add_packed(sum, own));
    return sum;
}

template <class O, bool QUEUE>
__global__ void __launch_bounds__(512) build_kernel(const DevParams p, const BuildArgs a)
{
    extern __shared__ __align__(16) uint8_t dyn_smem[];
    __shared__ SmemTables T;
    const int tid = threadIdx.x, nthr = blockDim.x;

    // ---- per-CTA setup: tables into shared memory ----
    for (int i = tid; i < 256 * 16; i += nthr) (&T.tri[0][0])[i] = (&UWW_TRI_TABLE[0][0])[i];
    for (int i = tid; i < 256; i += nthr) {
        T.edges[i] = UWW_CASE_EDGES[i];
        T.ntri[i] = UWW_CASE_NTRI[i];
        T.perm[i] = p.perm[i];
    }
    for (int i = tid; i < 12 * 4 * 5; i += nthr) (&T.share[0][0][0])[i] = (&UWW_EDGE_SHARE[0][0][0])[i];
    for (int i = tid; i < 24; i += nthr) (&T.corners[0][0])[i] = (&UWW_EDGE_CORNERS[0][0])[i];
    __syncthreads();
    // owned-edge mask for each boundary situation; cells of a chunk with N >= 2
    // only differ through the six "at a face" flags.
    for (int i = tid; i < 128; i += nthr) {
        const int oriented = i >> 6, f = i & 63;
        // a representative cell with these flags in a large chunk
        const int N = 4;
        const int x = (f & 1) ? 0 : ((f & 8) ? N - 1 : 1);
        const int y = (f & 2) ? 0 : ((f & 16) ? N - 1 : 1);
        const int z = (f & 4) ? 0 : ((f & 32) ? N - 1 : 1);
        unsigned m = 0;
        for (int e = 0; e < 12; ++e) {
            int ox, oy, oz;
            const int oe = find_owner(T, e, x, y, z, N, oriented != 0, ox, oy, oz);
            if (oe == e && ox == x && oy == y && oz == z) m |= 1u << e;
        }
        T.owned[oriented][f] = (uint16_t)m;
    }
    __syncthreads();

    const bool oriented = p.dedup_mode == UWW_DEDUP_ORIENTED;
    const bool want_color = (p.outputs & UWW_OUT_COLOR) != 0;
    const bool want_normals = (p.outputs & UWW_OUT_NORMALS) != 0 && a.normals != nullptr;
    const bool want_cases = (p.outputs & UWW_OUT_CASES) != 0 && a.cases != nullptr;

    for (;;) {
        if (tid == 0) T.ticket = QUEUE ? atomicAdd(a.work_counter, 1u) : 0u;
        __syncthreads();
        const uint32_t ticket = T.ticket;
        if (ticket >= a.n) break;

        const uww_chunk_desc d = a.chunks[ticket];
        const int N = (int)d.cells;
        const bool bad = N < 1 || N > (int)a.max_cells || N > UWW_MAX_CELLS;
        const int S = N + 1;
        const int NC = N * N * N;

        uint8_t* ws = nullptr;
        ChunkLayout L = chunk_layout(bad ? 1 : N);
        if (!bad) ws = (uint32_t)N <= a.smem_cells ? dyn_smem : a.scratch + (size_t)blockIdx.x * a.scratch_slot_bytes;
        float* rho = reinterpret_cast<float*>(ws + L.rho);
        uint8_t* cases = ws + L.cases;
        uint32_t* vbase = reinterpret_cast<uint32_t*>(ws + L.vbase);
        uint16_t* active16 = reinterpret_cast<uint16_t*>(ws + L.active);
        uint32_t* active32 = reinterpret_cast<uint32_t*>(ws + L.active);
        uint32_t* ibase = reinterpret_cast<uint32_t*>(ws + L.ibase);

        const int ox = d.pos[0] * p.chunk_size, oy = d.pos[1] * p.chunk_size, oz = d.pos[2] * p.chunk_size;

        // ---- 1. density grid (build_iso) + early blank vote ----
        int inside = 0;
        if (!bad) {
            const float s = __fdiv_rn((float)p.chunk_size, (float)N);  // SIZE_SCALE
            const int S2 = S * S, S3 = S2 * S;
            if (a.samples_in) {
                const float* src = a.samples_in + d.sample_offset;
                for (int idx = tid; idx < S3; idx += nthr) {
                    const float v = src[idx];
                    rho[idx] = v;
                    inside |= !(v > p.iso_level);
                }
            } else {
                for (int idx = tid; idx < S3; idx += nthr) {
                    const int x = idx / S2, r = idx - x * S2, y = r / S, z = r - y * S;
                    const float wx = O::add(O::mul((float)x, s), (float)ox);
                    const float wy = O::add(O::mul((float)y, s), (float)oy);
                    const float wz = O::add(O::mul((float)z, s), (float)oz);
                    const float v = density<O, false>(p, T.perm, wx, wy, wz, nullptr);
                    rho[idx] = v;
                    inside |= !(v > p.iso_level);
                }
            }
            if (a.samples_out) {
                float* dst = a.samples_out + d.sample_offset;
                for (int idx = tid; idx < S3; idx += nthr) dst[idx] = rho[idx];
            }
        }
        const int any_inside = __syncthreads_or(inside);

        unsigned long long total = 0ull;
        uint32_t flags = 0;
        if (bad) {
            if (tid == 0) atomicOr(&a.totals[3], kErrBadChunk);
        } else if (!any_inside) {
            flags = UWW_CHUNK_EARLY_BLANK;
            if (want_cases)
                for (int c = tid; c < NC; c += nthr) a.cases[(size_t)d.cell_offset + c] = 0;
        } else {
            // ---- 2. classify + count, contiguous runs of cells per thread ----
            const int R = (NC + nthr - 1) / nthr;
            const int c0 = min(tid * R, NC), c1 = min(c0 + R, NC);
            unsigned long long mine = 0ull;
            {
                int x = c0 / (N * N), y = (c0 / N) % N, z = c0 % N;
                for (int c = c0; c < c1; ++c) {
                    const int b = (x * S + y) * S + z;
                    const float iso = p.iso_level;
                    int cs = 0;
                    cs |= (rho[b] < iso) << 0;
                    cs |= (rho[b + S * S] < iso) << 1;
                    cs |= (rho[b + S * S + 1] < iso) << 2;
                    cs |= (rho[b + 1] < iso) << 3;
                    cs |= (rho[b + S] < iso) << 4;
                    cs |= (rho[b + S * S + S] < iso) << 5;
                    cs |= (rho[b + S * S + S + 1] < iso) << 6;
                    cs |= (rho[b + S + 1] < iso) << 7;
                    cases[c] = (uint8_t)cs;
                    const int nt = T.ntri[cs];
                    if (nt) {
                        const unsigned own = T.owned[oriented][boundary_flags(x, y, z, N)];
                        const unsigned nv = __popc(T.edges[cs] & own);
                        mine += (unsigned long long)nv | ((unsigned long long)(3 * nt) << kIndShift) |
                                (1ull << kActShift);
                    }
                    if (++z == N) { z = 0; if (++y == N) { y = 0; ++x; } }
                }
            }
            unsigned long long run = block_exclusive_scan(mine, T, total);
            {
                for (int c = c0; c < c1; ++c) {
                    const int cs = cases[c];
                    vbase[c] = (uint32_t)(run & kField22);
                    const int nt = T.ntri[cs];
                    if (nt) {
                        const uint32_t ar = (uint32_t)(run >> kActShift);
                        if (L.active16) active16[ar] = (uint16_t)c; else active32[ar] = (uint32_t)c;
                        ibase[ar] = (uint32_t)((run >> kIndShift) & kField22);
                        const int x = c / (N * N), y = (c / N) % N, z = c % N;
                        const unsigned own = T.owned[oriented][boundary_flags(x, y, z, N)];
                        run += (unsigned long long)__popc(T.edges[cs] & own) |
                               ((unsigned long long)(3 * nt) << kIndShift) | (1ull << kActShift);
                    }
                }
            }
            if (want_cases)
                for (int c = tid; c < NC; c += nthr) a.cases[(size_t)d.cell_offset + c] = cases[c];
        }

        const uint32_t nV = (uint32_t)(total & kField22);
        const uint32_t nI = (uint32_t)((total >> kIndShift) & kField22);
        const uint32_t nA = (uint32_t)(total >> kActShift);

        // ---- 3. output offsets ----
        if (tid < 32) {
            const unsigned long long own = (unsigned long long)nV | ((unsigned long long)nI << 30);
            unsigned long long ex = 0ull;
            if (QUEUE) ex = lookback(a, ticket, own);
            if (tid == 0) {
                const unsigned long long ev = ex & kLbVertMax, ei = (ex >> 30) & kLbIndMax;
                const bool fits = ev + nV <= a.vert_capacity && ei + nI <= a.ind_capacity;
                T.excl = ev | (ei << 32);
                T.fits = fits;
                if (nI > 0) flags |= UWW_CHUNK_HAS_MESH;
                if (!fits) {
                    flags |= UWW_CHUNK_OVERFLOW;
                    if (QUEUE) atomicAdd(&a.totals[2], 1ull);
                }
                uww_chunk_record rec;
                rec.num_verts = nV;
                rec.num_inds = nI;
                rec.vert_offset = (uint32_t)(ev > 0xffffffffull ? 0xffffffffull : ev);
                rec.ind_offset = (uint32_t)(ei > 0xffffffffull ? 0xffffffffull : ei);
                rec.flags = flags;
                rec.num_active_cells = nA;
                rec.reserved[0] = rec.reserved[1] = 0;
                a.records[ticket] = rec;
                if (!QUEUE) {
                    a.totals[0] = nV;
                    a.totals[1] = nI;
                    a.totals[2] = fits ? 0ull : 1ull;
                } else if (ticket == a.n - 1) {
                    a.totals[0] = ev + nV;
                    a.totals[1] = ei + nI;
                }
            }
        }
        __syncthreads();

        // ---- 4. emission ----
        if (!bad && any_inside && T.fits && nA > 0) {
            const uint32_t voff = (uint32_t)(T.excl & 0xffffffffull);
            const uint32_t ioff = (uint32_t)(T.excl >> 32);
            const float s = __fdiv_rn((float)p.chunk_size, (float)N);
            const float iso = p.iso_level;
            for (uint32_t ai = tid; ai < nA; ai += nthr) {
                const int c = L.active16 ? (int)active16[ai] : (int)active32[ai];
                const int x = c / (N * N), y = (c / N) % N, z = c % N;
                const int cs = cases[c];
                const int8_t* row = T.tri[cs];
                const unsigned own = T.owned[oriented][boundary_flags(x, y, z, N)];
                const uint32_t vb = vbase[c];
                const uint32_t ib = ibase[ai];
                unsigned seen = 0;
                uint32_t cnt = 0;
                const int nidx = 3 * T.ntri[cs];
                for (int i = 0; i < nidx; ++i) {
                    const int e = row[i];
                    const unsigned bit = 1u << e;
                    uint32_t id;
                    if (own & bit) {
                        if (!(seen & bit)) {
                            seen |= bit;
                            id = vb + cnt++;
                            // create the vertex (chunk.rs:176-231)
                            const int ca = T.corners[e][0], cb = T.corners[e][1];
                            const int ax = x + ((0x66 >> ca) & 1), ay = y + (ca >> 2), az = z + ((0xcc >> ca) & 1);
                            const int bx = x + ((0x66 >> cb) & 1), by = y + (cb >> 2), bz = z + ((0xcc >> cb) & 1);
                            const float ia = rho[(ax * S + ay) * S + az];
                            const float ibv = rho[(bx * S + by) * S + bz];
                            const float sax = O::mul((float)ax, s), say = O::mul((float)ay, s), saz = O::mul((float)az, s);
                            const float sbx = O::mul((float)bx, s), sby = O::mul((float)by, s), sbz = O::mul((float)bz, s);
                            const float t = __fdiv_rn(O::sub(iso, ia), O::sub(ibv, ia));
                            const float mx = O::add(sax, O::mul(t, O::sub(sbx, sax)));
                            const float my = O::add(say, O::mul(t, O::sub(sby, say)));
                            const float mz = O::add(saz, O::mul(t, O::sub(sbz, saz)));
                            const float wz = O::add(mz, (float)oz);
                            float pos[3] = {O::add(mx, (float)ox), O::add(my, (float)oy), wz};
                            float col[3] = {0.f, 0.f, 0.f};
                            if (want_color) vertex_color<O>(p, wz, cb, col);
                            uww_vert_color* vv = a.verts + voff + id;
                            float2* v2 = reinterpret_cast<float2*>(vv);
                            v2[0] = make_float2(pos[0], pos[1]);
                            v2[1] = make_float2(pos[2], col[0]);
                            v2[2] = make_float2(col[1], col[2]);
                            if (want_normals) {
                                float g[3];
                                density<O, true>(p, T.perm, pos[0], pos[1], pos[2], g);
                                safe_normalize<O>(g);
                                float* nn = a.normals + 3 * (size_t)(voff + id);
                                nn[0] = g[0]; nn[1] = g[1]; nn[2] = g[2];
                            }
                        } else {
                            id = vb + rank_in_row(row, own, e);
                        }
                    } else {
                        int qx, qy, qz;
                        const int oe = find_owner(T, e, x, y, z, N, oriented, qx, qy, qz);
                        const int oc = (qx * N + qy) * N + qz;
                        const unsigned oown = T.owned[oriented][boundary_flags(qx, qy, qz, N)];
                        id = vbase[oc] + rank_in_row(T.tri[cases[oc]], oown, oe);
                    }
                    a.inds[ioff + ib + i] = id;
                }
            }
        }
        if (!QUEUE) break;
        __syncthreads();  // the working set is reused by the next ticket
    }
}

template <class O>
__global__ void density_kernel(const DevParams p, const float* __restrict__ xyz, uint32_t n, float* __restrict__ out)
{
    __shared__ uint8_t P[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) P[i] = p.perm[i];
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = density<O, false>(p, P, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], nullptr);
}

template <class O, bool Q>
cudaError_t set_smem_attr(size_t bytes)
{
    return cudaFuncSetAttribute(build_kernel<O, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

size_t build_static_smem_bytes() { return sizeof(SmemTables); }

cudaError_t prepare_build_kernels(size_t max_dyn_smem)
{
    cudaError_t e;
    if ((e = set_smem_attr<ExactOps, true>(max_dyn_smem)) != cudaSuccess) return e;
    if ((e = set_smem_attr<ExactOps, false>(max_dyn_smem)) != cudaSuccess) return e;
    if ((e = set_smem_attr<FastOps, true>(max_dyn_smem)) != cudaSuccess) return e;
    return set_smem_attr<FastOps, false>(max_dyn_smem);
}

cudaError_t build_occupancy(bool queue, bool exact, int threads, size_t dyn_smem, int* blocks_per_sm)
{
    if (exact)
        return queue ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, build_kernel<ExactOps, true>, threads, dyn_smem)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, build_kernel<ExactOps, false>, threads, dyn_smem);
    return queue ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, build_kernel<FastOps, true>, threads, dyn_smem)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, build_kernel<FastOps, false>, threads, dyn_smem);
}

cudaError_t launch_build(const DevParams& p, const BuildArgs& a, bool queue, int grid, int threads, size_t dyn_smem,
                         cudaStream_t s)
{
    const bool exact = p.math_mode == UWW_MATH_EXACT;
    if (exact) {
        if (queue) build_kernel<ExactOps, true><<<grid, threads, dyn_smem, s>>>(p, a);
        else build_kernel<ExactOps, false><<<grid, threads, dyn_smem, s>>>(p, a);
    } else {
        if (queue) build_kernel<FastOps, true><<<grid, threads, dyn_smem, s>>>(p, a);
        else build_kernel<FastOps, false><<<grid, threads, dyn_smem, s>>>(p, a);
    }
    return cudaGetLastError();
}

cudaError_t launch_density(const DevParams& p, const float* xyz, uint32_t n, float* out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    const int grid = (int)((n + threads - 1) / threads);
    if (p.math_mode == UWW_MATH_EXACT) density_kernel<ExactOps><<<grid, threads, 0, s>>>(p, xyz, n, out);
    else density_kernel<FastOps><<<grid, threads, 0, s>>>(p, xyz, n, out);
    return cudaGetLastError();
}

}  // namespace uww
