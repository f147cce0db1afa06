// uww_build.cu -- the chunk-build kernel (noise + marching cubes + emission).
//
// One CTA builds one chunk at a time.  Per chunk:
//   front half (compute warps):
//     1. the (N+1)^3 density grid (Chunk::build_iso, chunk.rs:105-129) into
//        shared memory, and the early blank vote (chunk.rs:131-133);
//     2. each cell's 8-bit case (chunk.rs:144-162), its triangle count and the
//        number of vertices it creates, block-scanned in the reference's cell
//        order (x outer, y, z inner; chunk.rs:138-142);
//     3. publication of the chunk's counts for the device-wide prefix sum (a
//        decoupled look-back over the work-queue order);
//   back half:
//     4. the chunk's output offsets (control warp, from the look-back) and its
//        record;
//     5. emission (compute warps): pass 1, one thread per active cell, walks
//        the triangle rows (chunk.rs:164-251) and writes chunk-local u32
//        indices and vertex positions; pass 2, one thread per vertex, writes
//        the colour (chunk.rs:208-219) and the normal.
//
// Vertex dedup (chunk.rs:233) is resolved without a search: a crossed edge is
// referenced by every cell that holds it, so the vertex the reference creates
// for it is made by the first such cell in stream order (its "owner"), at the
// owner's first reference to that edge.  Vertex ids are the running count of
// owned first references, scanned over cells.
//
// Batched form: a persistent grid fed by a device work queue (an atomic ticket
// counter).  Each CTA is warp-specialised -- compute warps plus one control
// warp -- and pipelines two chunks: once the compute warps finish the noise of
// ticket i, the control warp resolves the look-back of ticket i-1 (while
// ticket i is classified), writes its record and takes ticket i+1 from the
// queue while ticket i-1 is emitted.  Look-back, record and ticket latency
// thus overlap compute.  The plain form (one chunk per launch) runs front then
// back with compute warps only.
//
// Planned batches: when neither samples nor cases are read or written, a
// one-CTA planning kernel (plan_kernel) first lists, in chunk order, the
// chunks the depth bias does not decide; the queue hands out only those, and
// the control warp of each listed chunk writes the records of the decided
// chunks that follow it (their offsets are its inclusive prefix).  A decided
// chunk thus costs a record write, not a ticket.
//
// Split form (the default batched build; the pipelined form above remains for
// samples read in, streamed host output and when asked for): three kernels,
// each the programmatic dependent of the one before.  split_plan_kernel
// decides what the depth bias decides and queues the rest, largest first;
// front_kernel (persistent, every thread a compute thread) runs steps 1-2 and
// pass 1 of each queued chunk into staging buffers and adds the chunk's counts
// to its tile's sum -- no look-back; emit_kernel writes the records from the
// tile sums, then takes blocks of staged vertices (pass 2) and of indices and
// stores them at their final offsets.  Chunks of 17..63 cells per edge are
// queued as x slabs of a few cell layers, one CTA each; a slab refers to the
// vertices of the previous slab's last layer through that slab's seam.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

// The tables live in global memory: every CTA copies them into shared memory
// once with coalesced loads (from the constant bank, per-thread addresses
// would be serialised).
#define UWW_TABLE_QUAL __device__
#include "mc_tables.h"
#include "uww_internal.h"
#include "uww_noise.cuh"

namespace uww {

namespace {

// Packed per-cell counts for the block scan: verts [21:0], inds [43:22], active [62:44].
constexpr int kIndShift = 22;
constexpr int kActShift = 44;
constexpr unsigned long long kField22 = (1ull << 22) - 1;
// split build: a chunk's counts word (tinfo) is the packed counts and, in
// bit 62, the early-blank flag
constexpr unsigned long long kInfoEarlyBlank = 1ull << 62;
// a meshed chunk the staging buffers had no room for
constexpr unsigned long long kUnstaged = ~0ull;
// emission units: kind in bits 60-62 (kUnitSlab: a slab of a large chunk,
// the slab in bits 48-59 and the part in 32-47), else the part in 32-59;
// the chunk in 0-31
constexpr uint32_t kUnitVerts = 0, kUnitInds = 1, kUnitChunk = 2, kUnitSlab = 8;
__device__ __forceinline__ unsigned long long unit_entry(uint32_t c, uint32_t part, uint32_t kind)
{
    return (unsigned long long)c | ((unsigned long long)part << 32) | ((unsigned long long)kind << 60);
}
__device__ __forceinline__ uint32_t rec_off32(unsigned long long v) { return (uint32_t)(v > 0xffffffffull ? 0xffffffffull : v); }



// Per in-flight chunk, kept in shared memory between the front and back halves.
struct ChunkInfo {
    uint32_t ticket;
    int32_t ox, oy, oz;
    int32_t N;
    uint32_t flags;               // UWW_CHUNK_EARLY_BLANK decided by the front half
    uint32_t classified;          // the mesh stage ran (not bad, not early blank)
    uint32_t chunk;               // index of the chunk in the batch (records are indexed by it)
    unsigned long long total;     // packed counts
};

struct Ticket {
    uww_chunk_desc desc;
    uint32_t ticket;              // position in the work queue (and of its look-back word)
    uint32_t chunk;               // the chunk it builds
    uint32_t pad[2];
};

struct Offsets {
    unsigned long long excl;      // verts | inds << 32
    uint32_t fits;
    uint32_t pad;
};

struct SmemTables {
    // the marching-cubes tables, the same for every parameter set (the
    // context's table image holds them)
    int8_t tri[256][16];
    uint16_t edges[256];
    uint16_t owned[2][64];        // [oriented?][boundary flags] -> owned edge mask
    uint16_t first_ref[256];      // per case: row positions that are their edge's first reference
    uint8_t ntri[256];
    uint8_t owner[2][8][12];      // UWW_EDGE_OWNER
    uint8_t corners[12][2];
    // the seeded permutation and its gradients
    float4 gp[256];               // gradient vector of P[i] (fast build: the last hash lookup)
    uint8_t perm[256];
    unsigned long long warp_sums[32];
    unsigned long long chunk_total;
    ChunkInfo ci[2];              // the chunks in flight (front / back)
    Ticket tk[2];                 // tickets handed from the control warp
    Offsets off[2];               // offsets handed from the control warp
    uint32_t overflow;            // chunks of this CTA that did not fit (control warp)
    uint32_t errflags;            // UWW_ERRFLAG_* raised by this CTA
    uint32_t last;                // this CTA is the last of the launch to finish
    uint32_t n;                   // tickets of this launch: the planned chunks, else every chunk
    uint32_t nchunks;             // chunks in this launch (min of the device count and BuildArgs::n)
};

// A cell's case from its four corner columns' inside masks (bit z: sample
// below the iso level), corner order of chunk.rs:144-153.
__device__ __forceinline__ int mask_case(unsigned long long m00, unsigned long long m10, unsigned long long m01,
                                         unsigned long long m11, int z)
{
    const unsigned long long z0 = m00 >> z, z1 = m10 >> z, z2 = m01 >> z, z3 = m11 >> z;
    return (int)((z0 & 1) | ((z1 & 1) << 1) | (((z1 >> 1) & 1) << 2) | (((z0 >> 1) & 1) << 3) | ((z2 & 1) << 4) |
                 ((z3 & 1) << 5) | (((z3 >> 1) & 1) << 6) | (((z2 >> 1) & 1) << 7));
}

__device__ __forceinline__ int boundary_flags(int x, int y, int z, int N)
{
    return (x == 0) | ((y == 0) << 1) | ((z == 0) << 2) | ((x == N - 1) << 3) | ((y == N - 1) << 4) |
           ((z == N - 1) << 5);
}


// ---------------------------------------------------------------------------
// The look-back words carry their own payload (no other data is published
// through them), so relaxed gpu-scope loads and stores suffice.
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Exclusive scan over the compute threads (ncomp, a multiple of 32).
__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v, SmemTables& T,
                                                                   unsigned long long& total, int ncomp)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = ncomp >> 5;
    unsigned long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) T.warp_sums[warp] = incl;
    bar_sync(kBarCompute, ncomp);
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
    bar_sync(kBarCompute, ncomp);
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

__device__ __forceinline__ unsigned long long pack_counts(unsigned long long total)
{
    return (total & kField22) | (((total >> kIndShift) & kField22) << 30);
}

// Publish a chunk's aggregate as soon as its counts are known (ticket 0
// publishes its inclusive prefix right away).
__device__ __forceinline__ void lookback_publish(const BuildArgs& a, uint32_t ticket, unsigned long long own)
{
    if (a.withhold_first && ticket == 0) return;  // failure injection: successors time out
    st_relaxed(&a.lookback[ticket], (ticket == 0 ? kLbInclusive : kLbAggregate) | own);
}

// Resolve a ticket's exclusive prefix, by one warp: sum the predecessors'
// words back to the nearest inclusive prefix (4 words per lane per round
// trip), then publish this ticket's inclusive prefix.  A predecessor that has
// not published yet, closer than the nearest inclusive prefix, means wait and
// re-read.  The wait is bounded by spin_limit_cycles; on timeout the prefix
// saturates (so nothing is written out of place) and the error flag is raised.
__device__ unsigned long long lookback_warp(const BuildArgs& a, uint32_t ticket, unsigned long long own,
                                           uint32_t* errflags)
{
    const int lane = threadIdx.x & 31;
    unsigned long long sum = 0ull;
    if (ticket > 0) {
        long long j = (long long)ticket - 1;
        const long long t0 = clock64();
        unsigned sleep_ns = 32;
        for (;;) {
            unsigned long long w[4];
            int mi = 0x7fffffff, mz = 0x7fffffff;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int dist = q * 32 + lane;
                const long long idx = j - dist;
                w[q] = idx >= 0 ? ld_relaxed(&a.lookback[idx]) : kLbInclusive;
                const unsigned st = (unsigned)(w[q] >> 62);
                if (st == 2u) mi = min(mi, dist);
                if (st == 0u) mz = min(mz, dist);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                mi = min(mi, __shfl_xor_sync(0xffffffffu, mi, o));
                mz = min(mz, __shfl_xor_sync(0xffffffffu, mz, o));
            }
            if (mz < mi) {  // an unpublished predecessor lies before the nearest inclusive prefix
                if (clock64() - t0 > a.spin_limit_cycles) {
                    if (lane == 0) atomicOr(errflags, (uint32_t)kErrTimeout);
                    sum = kLbVertMax | (kLbIndMax << 30);
                    break;
                }
                __nanosleep(sleep_ns);  // back off: the wait overlaps a noise phase
                sleep_ns = min(2u * sleep_ns, 512u);
                continue;
            }
            unsigned long long v = 0ull, i = 0ull;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q * 32 + lane <= mi) {
                    v += w[q] & kLbVertMax;
                    i += (w[q] >> 30) & kLbIndMax;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                v += __shfl_xor_sync(0xffffffffu, v, o);
                i += __shfl_xor_sync(0xffffffffu, i, o);
            }
            sum = sat_add_packed(sum, (v > kLbVertMax ? kLbVertMax : v) | ((i > kLbIndMax ? kLbIndMax : i) << 30));
            if (mi != 0x7fffffff) break;
            j -= 128;
        }
    }
    if (lane == 0 && !(a.withhold_first && ticket == 0))
        st_relaxed(&a.lookback[ticket], kLbInclusive | sat_add_packed(sum, own));
    return sum;
}

// The chunk record and its output offsets, from its exclusive prefix; run by
// one thread.
__device__ __forceinline__ void chunk_record(const BuildArgs& a, SmemTables& T, const ChunkInfo& ci,
                                             unsigned long long ex, Offsets& off, bool queue)
{
    const uint32_t nV = (uint32_t)(ci.total & kField22);
    const uint32_t nI = (uint32_t)((ci.total >> kIndShift) & kField22);
    const uint32_t nA = (uint32_t)(ci.total >> kActShift);
    const unsigned long long ev = ex & kLbVertMax, ei = (ex >> 30) & kLbIndMax;
    const bool fits = ev + nV <= a.vert_capacity && ei + nI <= a.ind_capacity;
    uint32_t flags = ci.flags;
    if (nI > 0) flags |= UWW_CHUNK_HAS_MESH;
    if (!fits) {
        flags |= UWW_CHUNK_OVERFLOW;
        T.overflow += 1;
    }
    off.excl = ev | (ei << 32);
    off.fits = fits;
    uww_chunk_record rec;
    rec.num_verts = nV;
    rec.num_inds = nI;
    rec.vert_offset = (uint32_t)(ev > 0xffffffffull ? 0xffffffffull : ev);
    rec.ind_offset = (uint32_t)(ei > 0xffffffffull ? 0xffffffffull : ei);
    rec.flags = flags;
    rec.num_active_cells = nA;
    rec.reserved[0] = rec.reserved[1] = 0;
    a.records[ci.chunk] = rec;
    if (a.host_records) a.host_records[ci.chunk] = rec;
    if (!queue || ci.ticket == T.n - 1) {
        a.totals[0] = ev + nV;
        a.totals[1] = ei + nI;
    }
}

// ---------------------------------------------------------------------------
struct Workspace {
    float* rho;
    uint8_t* cases;
    void* vbase;
    void* active;
    void* ibase;
    bool idx16, active16;
    __device__ uint32_t get_vbase(int c) const
    {
        return idx16 ? (uint32_t)reinterpret_cast<const uint16_t*>(vbase)[c] : reinterpret_cast<const uint32_t*>(vbase)[c];
    }
    __device__ void set_vbase(int c, uint32_t v) const
    {
        if (idx16) reinterpret_cast<uint16_t*>(vbase)[c] = (uint16_t)v; else reinterpret_cast<uint32_t*>(vbase)[c] = v;
    }
    __device__ uint32_t get_ibase(int i) const
    {
        return idx16 ? (uint32_t)reinterpret_cast<const uint16_t*>(ibase)[i] : reinterpret_cast<const uint32_t*>(ibase)[i];
    }
    __device__ void set_ibase(int i, uint32_t v) const
    {
        if (idx16) reinterpret_cast<uint16_t*>(ibase)[i] = (uint16_t)v; else reinterpret_cast<uint32_t*>(ibase)[i] = v;
    }
    __device__ int get_active(int i) const
    {
        return active16 ? (int)reinterpret_cast<const uint16_t*>(active)[i] : (int)reinterpret_cast<const uint32_t*>(active)[i];
    }
    __device__ void set_active(int i, int c) const
    {
        if (active16) reinterpret_cast<uint16_t*>(active)[i] = (uint16_t)c; else reinterpret_cast<uint32_t*>(active)[i] = (uint32_t)c;
    }
};

// Whether a chunk's emission finds each triangle's cell in a triangle map
// rather than by a search over its active cells: chunks of up to 16 cells per
// edge with 16-bit index positions and no more triangles than cells, whose
// map (x | y << 4 | z << 8 | row << 12 per triangle) fits in the ibase array.
__device__ __forceinline__ bool direct_triangles(const Workspace& W, int N, unsigned long long total)
{
    const uint32_t nT = (uint32_t)((total >> kIndShift) & kField22) / 3u;
    return N <= 16 && W.idx16 && nT <= (uint32_t)(N * N * N);
}

__device__ __forceinline__ Workspace workspace(const BuildArgs& a, uint8_t* dyn_smem, int buf, int N)
{
    const ChunkLayout L = chunk_layout(N);
    uint8_t* base = (uint32_t)N <= a.smem_cells
                        ? dyn_smem + (size_t)buf * a.smem_buf_bytes
                        : a.scratch + ((size_t)blockIdx.x * a.slots_per_cta + buf) * a.scratch_slot_bytes;
    Workspace w;
    w.rho = reinterpret_cast<float*>(base + L.rho);
    w.cases = base + L.cases;
    w.vbase = base + L.vbase;
    w.active = base + L.active;
    w.ibase = base + L.ibase;
    w.idx16 = L.idx16;
    w.active16 = L.active16;
    return w;
}

// Front half of a chunk into workspace `buf`.  Every compute thread must call it.
template <class O, bool QUEUE>
__device__ void chunk_front(const DevParams& p, const BuildArgs& a, SmemTables& T, uint8_t* dyn_smem,
                            const uww_chunk_desc d, uint32_t ticket, uint32_t chunk, int buf, int ncomp)
{
    const int tid = threadIdx.x;
    const int oriented = p.dedup_mode == UWW_DEDUP_ORIENTED;
    const bool want_cases = (p.outputs & UWW_OUT_CASES) != 0 && a.cases != nullptr;

    const bool cells_ok = d.cells >= 1 && d.cells <= a.max_cells && d.cells <= UWW_MAX_CELLS;
    const int N = cells_ok ? (int)d.cells : 1;
    const int S = N + 1;
    const int NC = N * N * N;
    // every global read or write of this chunk's per-cell / per-sample data
    // is checked against the capacity the caller gave
    const bool bad = !cells_ok ||
                     (a.samples_in && (unsigned long long)d.sample_offset + S * S * S > a.samples_in_count);
    const bool cases_ok = want_cases && !bad && (unsigned long long)d.cell_offset + NC <= a.case_capacity;
    const bool samples_ok = a.samples_out && !bad && (unsigned long long)d.sample_offset + S * S * S <= a.sample_capacity;
    if (tid == 0) {
        if (bad) atomicOr(&T.errflags, (uint32_t)kErrBadChunk);
        else if ((want_cases && !cases_ok) || (a.samples_out && !samples_ok)) atomicOr(&T.errflags, (uint32_t)kErrRange);
    }
    const Workspace W = workspace(a, dyn_smem, buf, N);
    float* rho = W.rho;
    uint8_t* cases = W.cases;
    const int ox = d.pos[0] * p.chunk_size, oy = d.pos[1] * p.chunk_size, oz = d.pos[2] * p.chunk_size;
    // a chunk in global scratch leaves the shared workspace `buf` free: its
    // columns' inside bits go there (fast build, up to 64 samples a column)
    // a 13^3-sample chunk in shared memory (register-column noise) writes
    // them to the mask area when the launch has one
    unsigned long long* masks =
        (std::is_same<O, FastOps>::value && (uint32_t)N > a.smem_cells && S <= 64 && !a.samples_in &&
         (size_t)S * S * sizeof(unsigned long long) <= a.smem_buf_bytes)
            ? reinterpret_cast<unsigned long long*>(dyn_smem + (size_t)buf * a.smem_buf_bytes)
        : (std::is_same<O, FastOps>::value && (uint32_t)N <= a.smem_cells && S == 13 && !a.samples_in &&
           a.mask_offset)
            ? reinterpret_cast<unsigned long long*>(dyn_smem + a.mask_offset)
            : nullptr;

    // ---- density grid (build_iso) + early blank and solid votes ----
    // A chunk whose depth bias keeps every sample above (below) the iso level
    // by more than the fBm can reach is blank (solid) without its noise --
    // unless its samples are read or written.
    const int decided = (!bad && !a.samples_in && !a.samples_out && !a.no_depth_shortcut) ? bias_decides(p, N, oz) : 0;
    int inside = decided == 2, outside = decided == 1;
    if (!bad && !decided) {
        const float s = __fdiv_rn((float)p.chunk_size, (float)N);  // SIZE_SCALE
        const int S2 = S * S, S3 = S2 * S;
        if (a.samples_in) {
            const float* src = a.samples_in + d.sample_offset;
            for (int idx = tid; idx < S3; idx += ncomp) {
                const float v = src[idx];
                rho[idx] = v;
                inside |= !(v > p.iso_level);
                outside |= !(v < p.iso_level);
            }
        } else if constexpr (std::is_same<O, FastOps>::value) {
            const ZTable zt = ztable_at(dyn_smem + a.ztable_offset, S, p.octaves);
            // the reference's 12^3 chunk accumulates its columns in registers; a
            // chunk in a global scratch slot accumulates them in local memory
            const bool in_smem = (uint32_t)N <= a.smem_cells;
            // (whole chunks do not settle early: on 12^3 chunks the checks
            // cost more than they save)
            const int io = (in_smem && S == 13)
                               ? sample_columns_reg<13>(p, T.perm, T.gp, zt, rho, ox, oy, oz, ncomp, masks)
                           : in_smem ? sample_columns_fast<false>(p, T.perm, T.gp, zt, rho, N, ox, oy, oz, ncomp)
                                     : sample_columns_fast<true>(p, T.perm, T.gp, zt, rho, N, ox, oy, oz, ncomp, masks);
            inside = io & 1;
            outside = io >> 1;
        } else {
            for (int idx = tid; idx < S3; idx += ncomp) {
                const int x = idx / S2, r = idx - x * S2, y = r / S, z = r - y * S;
                const float wx = O::add(O::mul((float)x, s), (float)ox);
                const float wy = O::add(O::mul((float)y, s), (float)oy);
                const float wz = O::add(O::mul((float)z, s), (float)oz);
                const float v = density<O, false>(p, T.perm, wx, wy, wz, nullptr);
                rho[idx] = v;
                inside |= !(v > p.iso_level);
                outside |= !(v < p.iso_level);
            }
        }
    }
    const int any_inside = bar_or(kBarCompute, ncomp, inside);
    // every sample below the iso level: every case is 255, no cell is
    // crossed, nothing to classify
    const int solid = bar_and(kBarCompute, ncomp, !outside);
    if (samples_ok) {
        float* dst = a.samples_out + d.sample_offset;
        for (int idx = tid; idx < S * S * S; idx += ncomp) dst[idx] = rho[idx];
    }

    unsigned long long total = 0ull;
    if (bad || !any_inside || solid) {
        if (QUEUE && tid == 0) lookback_publish(a, ticket, 0ull);
        if (!bad && cases_ok)
            for (int c = tid; c < NC; c += ncomp) a.cases[(size_t)d.cell_offset + c] = solid ? 255 : 0;
    } else {
        // ---- classify + count, contiguous runs of cells per thread: with
        // column masks and a thread for every column, a run is one column
        // (its quiet cells settled together by bit operations, its active
        // cells visited alone); else the cells split evenly ----
        const bool colrun = masks && N <= 16 && N * N <= ncomp && (uint32_t)N <= a.smem_cells;
        const int R = colrun ? N : (NC + ncomp - 1) / ncomp;
        const int c0 = min(tid * R, NC), c1 = min(c0 + R, NC);
        // up to 16 cells of a run keep their counts in registers for the
        // second pass, 8 bits a cell: triangles | new vertices << 3
        const bool keep = R <= 16;
        unsigned long long kept0 = 0ull, kept1 = 0ull;
        unsigned long long mine = 0ull;
        unsigned actbits = 0;  // (keep) bit i: cell c0 + i is active
        const int x0 = c0 / (N * N), y0 = (c0 / N) % N, z0 = c0 % N;
        if (colrun) {
            if (c0 < c1) {
                const int col = x0 * S + y0;
                const unsigned long long m00 = masks[col], m10 = masks[col + S], m01 = masks[col + 1],
                                         m11 = masks[col + S + 1];
                const unsigned long long an = m00 & m10 & m01 & m11, no = ~(m00 | m10 | m01 | m11);
                const unsigned long long allin = an & (an >> 1), quiet = allin | (no & (no >> 1));
                const unsigned long long cellbits = (1ull << N) - 1ull;
                if (cases_ok || !keep) {
                    // the quiet cells' cases are read (by the cases output)
                    for (int z = 0; z < N; ++z)
                        if ((quiet >> z) & 1ull) cases[c0 + z] = ((allin >> z) & 1ull) ? 255 : 0;
                }
                const unsigned own_lo = (x0 == 0) | ((y0 == 0) << 1) | ((x0 == N - 1) << 3) | ((y0 == N - 1) << 4);
                for (unsigned long long act = ~quiet & cellbits; act; act &= act - 1ull) {
                    const int z = __ffsll((long long)act) - 1;
                    const int cs = mask_case(m00, m10, m01, m11, z);
                    cases[c0 + z] = (uint8_t)cs;
                    const int nt = T.ntri[cs];
                    const unsigned own = T.owned[oriented][own_lo | ((z == 0) << 2) | ((z == N - 1) << 5)];
                    const unsigned nv = __popc(T.edges[cs] & own);
                    mine += (unsigned long long)nv | ((unsigned long long)(3 * nt) << kIndShift) | (1ull << kActShift);
                    const unsigned long long v = (unsigned long long)(nt | (nv << 3)) << (8 * (z & 7));
                    if (z < 8) kept0 |= v; else kept1 |= v;
                    actbits |= 1u << z;
                }
            }
        } else {
            int x = x0, y = y0, z = z0;
            const float iso = p.iso_level;
            const int SS = S * S;
            // the z+1 face of a cell is the z face of the next cell in the
            // run: carry its 4 inside bits (corners 3,2,7,6 -> 0,1,4,5)
            int lo = -1;
            unsigned long long m00 = 0, m10 = 0, m01 = 0, m11 = 0, quiet = 0, allin = 0;
            int mcol = -1;
            for (int c = c0; c < c1; ++c) {
                int cs;
                if (masks) {
                    // corner bits from the columns' masks (corner order of chunk.rs:144-153)
                    const int col = x * S + y;
                    if (col != mcol) {
                        m00 = masks[col]; m10 = masks[col + S]; m01 = masks[col + 1]; m11 = masks[col + S + 1];
                        mcol = col;
                        // bit z: cell z has all eight corners below (allin) or
                        // all above-or-at the iso level -- case 255 or 0
                        const unsigned long long an = m00 & m10 & m01 & m11, no = ~(m00 | m10 | m01 | m11);
                        allin = an & (an >> 1);
                        quiet = allin | (no & (no >> 1));
                    }
                    if ((quiet >> z) & 1ull) {
                        cases[c] = ((allin >> z) & 1ull) ? 255 : 0;
                        if (++z == N) { z = 0; if (++y == N) { y = 0; ++x; } }
                        continue;
                    }
                    cs = mask_case(m00, m10, m01, m11, z);
                } else {
                    const int b = (x * S + y) * S + z;
                    if (lo < 0)
                        lo = (rho[b] < iso) | ((rho[b + SS] < iso) << 1) | ((rho[b + S] < iso) << 4) |
                             ((rho[b + SS + S] < iso) << 5);
                    const int c3 = rho[b + 1] < iso, c2 = rho[b + SS + 1] < iso;
                    const int c7 = rho[b + S + 1] < iso, c6 = rho[b + SS + S + 1] < iso;
                    cs = lo | (c2 << 2) | (c3 << 3) | (c6 << 6) | (c7 << 7);
                    lo = (z + 1 < N) ? (c3 | (c2 << 1) | (c7 << 4) | (c6 << 5)) : -1;
                }
                cases[c] = (uint8_t)cs;
                const int nt = T.ntri[cs];
                if (nt) {
                    const unsigned own = T.owned[oriented][boundary_flags(x, y, z, N)];
                    const unsigned nv = __popc(T.edges[cs] & own);
                    mine += (unsigned long long)nv | ((unsigned long long)(3 * nt) << kIndShift) | (1ull << kActShift);
                    if (keep) {
                        const int i = c - c0;
                        const unsigned long long v = (unsigned long long)(nt | (nv << 3)) << (8 * (i & 7));
                        if (i < 8) kept0 |= v; else kept1 |= v;
                        actbits |= 1u << i;
                    }
                }
                if (++z == N) { z = 0; if (++y == N) { y = 0; ++x; } }
            }
        }
        unsigned long long run = block_exclusive_scan(mine, T, total, ncomp);
        // publish the aggregate as soon as the counts are known
        if (QUEUE && tid == 0) lookback_publish(a, ticket, pack_counts(total));
        const bool direct = direct_triangles(W, N, total);
        // second pass over the same runs: each active cell's first vertex id
        // (only active cells need one: every owner cell of a crossed edge is
        // active) and where its triangles go -- the triangle map (direct),
        // else the active-cell list with first index positions
        auto place = [&](int c, int x, int y, int z, int nt, unsigned nv) {
            W.set_vbase(c, (uint32_t)(run & kField22));
            const uint32_t ir = (uint32_t)((run >> kIndShift) & kField22);
            if (direct) {
                uint16_t* tmap = reinterpret_cast<uint16_t*>(W.ibase) + ir / 3u;
                const unsigned xyz = (unsigned)x | ((unsigned)y << 4) | ((unsigned)z << 8);
                for (int k = 0; k < nt; ++k) tmap[k] = (uint16_t)(xyz | ((unsigned)k << 12));
            } else {
                const uint32_t ar = (uint32_t)(run >> kActShift);
                W.set_active(ar, c);
                W.set_ibase(ar, ir);
            }
            run += (unsigned long long)nv | ((unsigned long long)(3 * nt) << kIndShift) | (1ull << kActShift);
        };
        if (keep) {
            // the active cells of the run, in order, from the kept counts
            for (unsigned bits = actbits; bits; bits &= bits - 1) {
                const int i = __ffs(bits) - 1;
                int x = x0, y = y0, z = z0 + i;
                while (z >= N) { z -= N; if (++y == N) { y = 0; ++x; } }
                const unsigned v = (unsigned)(((i < 8 ? kept0 : kept1) >> (8 * (i & 7))) & 0xffu);
                place(c0 + i, x, y, z, (int)(v & 7u), v >> 3);
            }
        } else {
            int x = x0, y = y0, z = z0;
            unsigned long long m00 = 0, m10 = 0, m01 = 0, m11 = 0;
            int mcol = -1;
            for (int c = c0; c < c1; ++c) {
                int cs;
                if (masks) {
                    // the case again from the masks (no read of the global cases)
                    const int col = x * S + y;
                    if (col != mcol) {
                        m00 = masks[col]; m10 = masks[col + S]; m01 = masks[col + 1]; m11 = masks[col + S + 1];
                        mcol = col;
                    }
                    cs = mask_case(m00, m10, m01, m11, z);
                } else {
                    cs = cases[c];
                }
                const int nt = T.ntri[cs];
                if (nt) place(c, x, y, z, nt, __popc(T.edges[cs] & T.owned[oriented][boundary_flags(x, y, z, N)]));
                if (++z == N) { z = 0; if (++y == N) { y = 0; ++x; } }
            }
        }
        if (cases_ok)
            for (int c = tid; c < NC; c += ncomp) a.cases[(size_t)d.cell_offset + c] = cases[c];
    }
    if (tid == 0) {
        ChunkInfo& ci = T.ci[buf];
        ci.ticket = ticket;
        ci.chunk = chunk;
        ci.ox = ox; ci.oy = oy; ci.oz = oz;
        ci.N = N;
        ci.flags = (!bad && !any_inside) ? UWW_CHUNK_EARLY_BLANK : 0u;
        ci.classified = !bad && any_inside;
        ci.total = total;
    }
}

// Pass 2 of the emission for vertex v: pass 1 left its position and, in
// colour slot 0, the owner's corner b (the value ramp's input, chunk.rs:215);
// write its colour and unit normal.
template <class O>
__device__ __forceinline__ void vertex_values(const DevParams& p, const uint8_t* P, const float4* gp, float2 p01,
                                              float2 p2c, bool want_color, bool want_normals, float2 out[3],
                                              float g[3])
{
    const int cb = (int)p2c.y;
    out[0] = p01;
    if (want_color) {
        float col[3];
        vertex_color<O>(p, p2c.x, cb, col);
        out[1] = make_float2(p2c.x, col[0]);
        out[2] = make_float2(col[1], col[2]);
    } else {
        out[1] = make_float2(p2c.x, 0.f);
        out[2] = make_float2(0.f, 0.f);
    }
    if (want_normals) {
        if constexpr (std::is_same<O, FastOps>::value)
            density_grad_fast(p, P, gp, p01.x, p01.y, p2c.x, g);
        else
            density<O, true>(p, P, p01.x, p01.y, p2c.x, g);
        safe_normalize<O>(g);
    }
}

template <class O>
__device__ __forceinline__ void vertex_outputs(const DevParams& p, const uint8_t* P, const float4* gp,
                                               const uww_vert_color* verts, uint32_t v, bool want_color,
                                               bool want_normals, float2 out[3], float g[3])
{
    // position and carried corner from L2: written by another thread of the
    // batch (pass 1), in this grid or the one before it
    const float2* v2 = reinterpret_cast<const float2*>(verts + v);
    vertex_values<O>(p, P, gp, __ldcg(v2), __ldcg(v2 + 1), want_color, want_normals, out, g);
}

template <class O>
__device__ __forceinline__ void finish_vertex(const DevParams& p, const uint8_t* P, const float4* gp,
                                              uww_vert_color* verts, float* normals, uint32_t v, bool want_color,
                                              bool want_normals)
{
    float2 out[3];
    float g[3];
    vertex_outputs<O>(p, P, gp, verts, v, want_color, want_normals, out, g);
    float2* v2 = reinterpret_cast<float2*>(verts + v);
    v2[1] = out[1];
    v2[2] = out[2];
    if (want_normals) {
        float* nn = normals + 3 * (size_t)v;
        nn[0] = g[0]; nn[1] = g[1]; nn[2] = g[2];
    }
}

// The vertex on edge e of cell (x, y, z): its chunk-local position (plus
// the chunk origin ox, oy, oz), the cell's corner b of the edge (the colour
// ramp's input) and, for the adjoint, its edge id (first-corner sample index
// << 3 | direction of corner b from corner a: +x -x +y -y +z -z).
struct EdgeVertex {
    float x, y, z;
    int cb;
    uint32_t edge_id;
};

// (rho holds the x planes from xo on: a slab's samples)
template <class O>
__device__ __forceinline__ EdgeVertex edge_vertex(const DevParams& p, const SmemTables& T, const float* rho, int S,
                                                  int x, int y, int z, int e, float s, int ox, int oy, int oz,
                                                  int xo = 0)
{
    const float iso = p.iso_level;
    const int ca = T.corners[e][0], cb = T.corners[e][1];
    const int ax = x + ((0x66 >> ca) & 1), ay = y + (ca >> 2), az = z + ((0xcc >> ca) & 1);
    const int bx = x + ((0x66 >> cb) & 1), by = y + (cb >> 2), bz = z + ((0xcc >> cb) & 1);
    const float ia = rho[((ax - xo) * S + ay) * S + az];
    const float ibv = rho[((bx - xo) * S + by) * S + bz];
    const float sax = O::mul((float)ax, s), say = O::mul((float)ay, s), saz = O::mul((float)az, s);
    const float sbx = O::mul((float)bx, s), sby = O::mul((float)by, s), sbz = O::mul((float)bz, s);
    const float tt = O::div(O::sub(iso, ia), O::sub(ibv, ia));
    const float mx = O::add(sax, O::mul(tt, O::sub(sbx, sax)));
    const float my = O::add(say, O::mul(tt, O::sub(sby, say)));
    const float mz = O::add(saz, O::mul(tt, O::sub(sbz, saz)));
    EdgeVertex v;
    v.x = O::add(mx, (float)ox);
    v.y = O::add(my, (float)oy);
    v.z = O::add(mz, (float)oz);
    v.cb = cb;
    const int dir = bx != ax ? (bx < ax) : by != ay ? 2 + (by < ay) : 4 + (bz < az);
    v.edge_id = ((uint32_t)((ax * S + ay) * S + az) << 3) | (uint32_t)dir;
    return v;
}

// Where pass 1 writes: the batch's outputs, or the split build's staging
// buffers.
struct EmitOut {
    uww_vert_color* verts;
    uint32_t* inds;
    uint32_t* edge_ids;
    float4* pos;  // when set: position and corner b per vertex instead of verts (staged pass 1)
};

// Pass 1 for triangle t of a chunk's index stream: its cell from the
// triangle map (else a binary search over the active cells), its three
// chunk-local vertex ids into inds, and the positions of the vertices its
// cell creates (the first reference of an owned edge).  The workspace W is
// in shared memory or a scratch slot (the build kernel); the arithmetic is the
// same either way.
// carry_corner: pass 2 follows, and colour slot 0 carries the owner's corner b.
// positions: write the vertices the cell creates (the split build's vertex
// work writes them instead).
template <class O>
__device__ __forceinline__ void emit_triangle(const DevParams& p, const EmitOut& a, const SmemTables& T,
                                              const Workspace& W, int N, uint32_t nA, bool direct, uint32_t t,
                                              uint32_t voff, uint32_t ioff, int ox, int oy, int oz, float s,
                                              bool carry_corner, bool positions = true)
{
    const int oriented = p.dedup_mode == UWW_DEDUP_ORIENTED;
    const int S = N + 1;
    const float* rho = W.rho;
    const uint8_t* cases = W.cases;
    const uint32_t g = 3u * t;
    int c, x, y, z, j0;
    if (direct) {
        const unsigned e = reinterpret_cast<const uint16_t*>(W.ibase)[t];
        x = (int)(e & 15u);
        y = (int)((e >> 4) & 15u);
        z = (int)((e >> 8) & 15u);
        j0 = 3 * (int)(e >> 12);
        c = (x * N + y) * N + z;
    } else {
        uint32_t ai = 0, len = nA;
        while (len > 1) {
            const uint32_t h = len >> 1;
            if (W.get_ibase(ai + h) <= g) ai += h;
            len -= h;
        }
        c = W.get_active(ai);
        x = c / (N * N);
        y = (c / N) % N;
        z = c % N;
        j0 = (int)(g - W.get_ibase(ai));
    }
    const int cs = cases[c];
    const int8_t* row = T.tri[cs];
    const unsigned own_mask = T.owned[oriented][boundary_flags(x, y, z, N)];
    const unsigned fr = T.first_ref[cs];
    const uint32_t vb = W.get_vbase(c);
    const uint16_t* before = UWW_EDGE_BEFORE[cs];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const int i = j0 + m;
        const int e = row[i];
        const unsigned bit = 1u << e;
        uint32_t id;
        if (own_mask & bit) {
            // the cell numbers its owned edges' vertices in first-reference order
            id = vb + __popc(own_mask & __ldg(before + e));
            if (positions && ((fr >> i) & 1u)) {
                const EdgeVertex ev = edge_vertex<O>(p, T, rho, S, x, y, z, e, s, ox, oy, oz);
                if (a.edge_ids) a.edge_ids[voff + id] = ev.edge_id;
                if (a.pos) {
                    a.pos[voff + id] = make_float4(ev.x, ev.y, ev.z, (float)ev.cb);
                } else {
                    float2* v2 = reinterpret_cast<float2*>(a.verts + voff + id);
                    v2[0] = make_float2(ev.x, ev.y);
                    // colour slot 0 carries the owner's corner b (the value
                    // ramp's input, chunk.rs:215) to pass 2, which overwrites it
                    v2[1] = make_float2(ev.z, carry_corner ? (float)ev.cb : 0.f);
                    v2[2] = make_float2(0.f, 0.f);
                }
            }
        } else {
            // the owner: the first cell in stream order holding this edge
            const int ow = T.owner[oriented][(x == 0) | ((y == 0) << 1) | ((z == 0) << 2)][e];
            const int qx = x - ((ow >> 4) & 1), qy = y - ((ow >> 5) & 1), qz = z - ((ow >> 6) & 1);
            const int oe = ow & 15;
            const int oc = (qx * N + qy) * N + qz;
            const unsigned oown = T.owned[oriented][boundary_flags(qx, qy, qz, N)];
            id = W.get_vbase(oc) + __popc(oown & __ldg(&UWW_EDGE_BEFORE[cases[oc]][oe]));
        }
        a.inds[ioff + g + m] = id;
    }
}

// Copy n 32-bit words, by threads tid, tid + nt, ...: 16-byte words where
// dst and src sit at the same offset from a 16-byte boundary, single words
// otherwise.  Used for output bound for page-locked host memory, where wide
// stores make the fewest transfers.
__device__ __forceinline__ void copy_words(uint32_t* dst, const uint32_t* src, uint32_t n, int tid, int nt)
{
    uint32_t head = n;
    if ((((uintptr_t)dst ^ (uintptr_t)src) & 15) == 0)
        head = min(n, (uint32_t)((16 - ((uintptr_t)src & 15)) & 15) / 4);
    for (uint32_t i = tid; i < head; i += nt) dst[i] = src[i];
    const uint32_t n4 = (n - head) / 4;
    const uint4* s4 = reinterpret_cast<const uint4*>(src + head);
    uint4* d4 = reinterpret_cast<uint4*>(dst + head);
    for (uint32_t i = tid; i < n4; i += nt) d4[i] = s4[i];
    for (uint32_t i = head + 4 * n4 + tid; i < n; i += nt) dst[i] = src[i];
}

// Emission of a chunk from workspace `buf`, given its offsets.  Every compute
// thread must call it.
template <class O, bool QUEUE>
__device__ void chunk_emit(const DevParams& p, const BuildArgs& a, SmemTables& T, uint8_t* dyn_smem, int buf,
                           const Offsets off, int ncomp)
{
    const int tid = threadIdx.x;
    const ChunkInfo ci = T.ci[buf];
    const uint32_t nV = (uint32_t)(ci.total & kField22);
    const uint32_t nA = (uint32_t)(ci.total >> kActShift);
    if (!(ci.classified && off.fits && nA > 0)) return;
    const bool want_color = (p.outputs & UWW_OUT_COLOR) != 0;
    const bool want_normals = (p.outputs & UWW_OUT_NORMALS) != 0 && a.normals != nullptr;
    const int N = ci.N;
    const uint32_t voff = (uint32_t)(off.excl & 0xffffffffull);
    const uint32_t ioff = (uint32_t)(off.excl >> 32);
    const Workspace W = workspace(a, dyn_smem, buf, N);
    const int ox = ci.ox, oy = ci.oy, oz = ci.oz;
    {
        const float s = __fdiv_rn((float)p.chunk_size, (float)N);
        // one thread per triangle of the chunk's index stream, so a dense
        // chunk's emission is spread over the CTA like a sparse one's; a
        // triangle's cell is the last active cell whose first index position
        // is at or before it
        const uint32_t nT = (uint32_t)((ci.total >> kIndShift) & kField22) / 3u;
        const bool direct = direct_triangles(W, N, ci.total);
        for (uint32_t t = tid; t < nT; t += ncomp)
            emit_triangle<O>(p, EmitOut{a.verts, a.inds, a.edge_ids}, T, W, N, nA, direct, t, voff, ioff, ox, oy, oz, s,
                             want_color || want_normals);
    }
    // pass 2 (colour and normal per vertex): inline for one chunk per launch
    // and for streamed host output; otherwise the batched form runs it as
    // vertex_kernel over the whole batch
    const bool stream_host = QUEUE && a.host_verts != nullptr;
    if ((!QUEUE || stream_host) && (want_color || want_normals)) {
        bar_sync(kBarCompute, ncomp);
        for (uint32_t vid = tid; vid < nV; vid += ncomp)
            finish_vertex<O>(p, T.perm, T.gp, a.verts, a.normals, voff + vid, want_color, want_normals);
    }
    // streamed host output: the finished chunk, just written by this CTA,
    // goes on to host memory in 16-byte words while later chunks build
    if (stream_host) {
        bar_sync(kBarCompute, ncomp);
        const uint32_t nI = (uint32_t)((ci.total >> kIndShift) & kField22);
        copy_words(a.host_inds + ioff, a.inds + ioff, nI, tid, ncomp);
        copy_words(reinterpret_cast<uint32_t*>(a.host_verts + voff), reinterpret_cast<const uint32_t*>(a.verts + voff),
                   6 * nV, tid, ncomp);
        if (want_normals && a.host_normals)
            copy_words(reinterpret_cast<uint32_t*>(a.host_normals + 3 * (size_t)voff),
                       reinterpret_cast<const uint32_t*>(a.normals + 3 * (size_t)voff), 3 * nV, tid, ncomp);
    }
}

// Control warp: take a ticket from the work queue and stage its chunk's
// descriptor (the planned chunk list maps tickets to chunks).
__device__ __forceinline__ void take_ticket(const BuildArgs& a, uint32_t n, Ticket& tk)
{
    const int lane = threadIdx.x & 31;
    uint32_t t = 0, c = 0;
    if (lane == 0) {
        t = atomicAdd(a.work_counter, 1u);
        c = (a.plan && t < n) ? __ldcg(&a.plan[kPlanList + t]) : t;
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (t < n && lane < 8)
        reinterpret_cast<uint32_t*>(&tk.desc)[lane] = reinterpret_cast<const uint32_t*>(&a.chunks[c])[lane];
    if (lane == 0) {
        tk.ticket = t;
        tk.chunk = c;
    }
    __syncwarp();
}

// The record of chunk j, which the depth bias decided (kind 1: every sample
// above the iso level, early blank; 2: every sample below it): no vertices,
// no indices, offsets at the prefix (ev, ei).  Returns whether it fits.
__device__ __forceinline__ bool decided_record(const BuildArgs& a, uint32_t j, int kind, unsigned long long ev,
                                               unsigned long long ei)
{
    const bool fits = ev <= a.vert_capacity && ei <= a.ind_capacity;
    uww_chunk_record rec;
    rec.num_verts = 0;
    rec.num_inds = 0;
    rec.vert_offset = (uint32_t)(ev > 0xffffffffull ? 0xffffffffull : ev);
    rec.ind_offset = (uint32_t)(ei > 0xffffffffull ? 0xffffffffull : ei);
    rec.flags = (kind == 1 ? UWW_CHUNK_EARLY_BLANK : 0u) | (fits ? 0u : UWW_CHUNK_OVERFLOW);
    rec.num_active_cells = 0;
    rec.reserved[0] = rec.reserved[1] = 0;
    a.records[j] = rec;
    if (a.host_records) a.host_records[j] = rec;
    return fits;
}

// Control warp, planned batches: the records of the decided chunks
// [lo, hi) that follow a listed chunk, at that chunk's inclusive prefix.
__device__ void decided_tail(const DevParams& p, const BuildArgs& a, SmemTables& T, uint32_t lo, uint32_t hi,
                             unsigned long long incl)
{
    const int lane = threadIdx.x & 31;
    const unsigned long long ev = incl & kLbVertMax, ei = (incl >> 30) & kLbIndMax;
    uint32_t over = 0;
    for (uint32_t j = lo + lane; j < hi; j += 32) {
        const uww_chunk_desc d = a.chunks[j];
        const int kind = bias_decides(p, (int)d.cells, d.pos[2] * p.chunk_size);
        over += decided_record(a, j, kind, ev, ei) ? 0u : 1u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) over += __shfl_xor_sync(0xffffffffu, over, o);
    if (lane == 0) T.overflow += over;
}

// Per-CTA setup: the marching-cubes tables, the permutation and its gradient
// table into shared memory (coalesced loads from global memory; per-thread
// addresses into the constant bank would be serialised).  The caller
// synchronises the CTA before use.
__device__ __forceinline__ void load_tables(const DevParams& p, SmemTables& T, int tid, int nthr)
{
    {
        const int4* src = reinterpret_cast<const int4*>(&UWW_TRI_TABLE[0][0]);
        int4* dst = reinterpret_cast<int4*>(&T.tri[0][0]);
        for (int i = tid; i < 256; i += nthr) dst[i] = __ldg(src + i);
    }
    for (int i = tid; i < 256; i += nthr) {
        T.edges[i] = __ldg(&UWW_CASE_EDGES[i]);
        T.ntri[i] = __ldg(&UWW_CASE_NTRI[i]);
    }
    // the permutation arrives in the parameter (constant) bank: read it as words
    for (int i = tid; i < 64; i += nthr) reinterpret_cast<uint32_t*>(T.perm)[i] = reinterpret_cast<const uint32_t*>(p.perm)[i];
    for (int i = tid; i < 128; i += nthr) (&T.owned[0][0])[i] = __ldg(&UWW_OWNED_MASK[0][0] + i);
    for (int i = tid; i < 2 * 8 * 12; i += nthr) (&T.owner[0][0][0])[i] = __ldg(&UWW_EDGE_OWNER[0][0][0] + i);
    for (int i = tid; i < 24; i += nthr) (&T.corners[0][0])[i] = __ldg(&UWW_EDGE_CORNERS[0][0] + i);
    __syncthreads();
    for (int cs = tid; cs < 256; cs += nthr) {
        unsigned seen = 0, fr = 0;
        for (int i = 0; i < 15 && T.tri[cs][i] >= 0; ++i) {
            const unsigned bit = 1u << T.tri[cs][i];
            if (!(seen & bit)) fr |= 1u << i;
            seen |= bit;
        }
        T.first_ref[cs] = (uint16_t)fr;
    }
    for (int i = tid; i < 256; i += nthr) {
        float gx, gy, gz;
        grad_vec(T.perm[i], gx, gy, gz);
        T.gp[i] = make_float4(gx, gy, gz, 0.f);
    }
}

// The marching-cubes part of SmemTables (everything before the permutation)
// as one image, built once per context by table_image_kernel and copied by
// each CTA in 8-byte words -- one round of coalesced loads instead of the
// table loads and their derivation; the permutation and its gradients come
// from the kernel parameters (64 threads, four entries each).
constexpr size_t kTableImageBytes = offsetof(SmemTables, gp);
static_assert(kTableImageBytes % 8 == 0, "the table image is copied in 8-byte words");

__device__ __forceinline__ void load_tables_image(const DevParams& p, const BuildArgs& a, SmemTables& T, int tid,
                                                  int nthr)
{
    if (!a.tables) {
        load_tables(p, T, tid, nthr);
        return;
    }
    uint2* dst = reinterpret_cast<uint2*>(&T);
    for (int i = tid; i < (int)(kTableImageBytes / 8); i += nthr) dst[i] = __ldg(a.tables + i);
    for (int i = tid; i < 64; i += nthr) {
        const uint32_t w = reinterpret_cast<const uint32_t*>(p.perm)[i];
        reinterpret_cast<uint32_t*>(T.perm)[i] = w;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float gx, gy, gz;
            grad_vec((int)((w >> (8 * k)) & 255u), gx, gy, gz);
            T.gp[4 * i + k] = make_float4(gx, gy, gz, 0.f);
        }
    }
}

__global__ void __launch_bounds__(256) table_image_kernel(const DevParams p, uint2* out)
{
    __shared__ SmemTables T;
    load_tables(p, T, threadIdx.x, blockDim.x);
    __syncthreads();
    const uint2* src = reinterpret_cast<const uint2*>(&T);
    for (int i = threadIdx.x; i < (int)(kTableImageBytes / 8); i += blockDim.x) out[i] = src[i];
}

// MAXT/MINB: the launch bounds of an instantiation.  Chunks of up to 16 cells
// per edge run with <= 224 threads (192 compute + the control warp) and at
// least 4 CTAs per SM (<= 72
// registers); larger chunks run with up to 544 threads.
template <class O, bool QUEUE, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) build_kernel(const DevParams p, const BuildArgs a)
{
    extern __shared__ __align__(16) uint8_t dyn_smem[];
    __shared__ SmemTables T;
    const int tid = threadIdx.x, nthr = blockDim.x;
    // batched form: the last warp is the control warp
    const int ncomp = QUEUE ? nthr - 32 : nthr;

    load_tables_image(p, a, T, tid, nthr);
    // a planned batch reads the chunk list of the planning kernel launched
    // just before it (as a programmatic dependent: the table setup above
    // overlaps the planning)
    if (QUEUE && a.plan) asm volatile("griddepcontrol.wait;" ::: "memory");
    // the vertex pass, launched after this kernel as its programmatic
    // dependent, may take SMs as this kernel's CTAs finish (it waits for the
    // whole build before reading anything)
    if (QUEUE) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (tid == 0) {
        T.errflags = 0;
        T.overflow = 0;
        T.nchunks = a.n_dev ? min(*a.n_dev, a.n) : a.n;
        T.n = (QUEUE && a.plan) ? __ldcg(&a.plan[kPlanCount]) : T.nchunks;
    }
    __syncthreads();

    if (!QUEUE) {
        chunk_front<O, QUEUE>(p, a, T, dyn_smem, a.chunks[0], 0u, 0u, 0, ncomp);
        bar_sync(kBarCompute, ncomp);
        if (tid == 0) chunk_record(a, T, T.ci[0], 0ull, T.off[0], false);
        bar_sync(kBarCompute, ncomp);
        chunk_emit<O, QUEUE>(p, a, T, dyn_smem, 0, T.off[0], ncomp);
        bar_sync(kBarCompute, ncomp);
        if (tid == 0) {
            a.totals[2] = T.overflow;
            a.totals[3] = T.errflags;
        }
        return;
    }

    if (tid >= ncomp) {
        // ---- control warp ----
        take_ticket(a, T.n, T.tk[0]);
        for (int i = 0;; ++i) {
            bar_sync(kBarTicket, nthr);  // ticket i staged; chunk i-1's counts visible
            const bool valid = T.tk[i & 1].ticket < T.n;
            // the look-back of chunk i-1 runs while the compute warps sample
            // chunk i, so its offsets are ready when they finish chunk i's
            // front half
            if (i > 0) {
                const ChunkInfo ci = T.ci[(i - 1) & 1];
                const unsigned long long own = pack_counts(ci.total);
                const unsigned long long ex = lookback_warp(a, ci.ticket, own, &T.errflags);
                if ((tid & 31) == 0) chunk_record(a, T, ci, ex, T.off[(i - 1) & 1], true);
                __syncwarp();
                bar_sync(kBarOffsets, nthr);
                if (a.plan) {
                    // the decided chunks up to the next listed one
                    const uint32_t next = ci.ticket + 1 < T.n ? __ldcg(&a.plan[kPlanList + ci.ticket + 1]) : T.nchunks;
                    decided_tail(p, a, T, ci.chunk + 1, next, sat_add_packed(ex, own));
                }
            }
            if (!valid) break;
            // the next ticket, while chunk i-1 is emitted
            take_ticket(a, T.n, T.tk[(i + 1) & 1]);
        }
    } else {
        // ---- compute warps ----
        for (int i = 0;; ++i) {
            bar_sync(kBarTicket, nthr);
            const Ticket tk = T.tk[i & 1];
            const bool valid = tk.ticket < T.n;
            if (valid) chunk_front<O, QUEUE>(p, a, T, dyn_smem, tk.desc, tk.ticket, tk.chunk, i & 1, ncomp);
            bar_sync(kBarCompute, ncomp);
            if (i > 0) {
                bar_sync(kBarOffsets, nthr);
                chunk_emit<O, QUEUE>(p, a, T, dyn_smem, (i - 1) & 1, T.off[(i - 1) & 1], ncomp);
                bar_sync(kBarCompute, ncomp);  // workspace (i-1)&1 is reused by chunk i+1
            }
            if (!valid) break;
        }
    }

    // ---- end of launch: fold this CTA's counters; the last CTA publishes
    // them and leaves the look-back state zeroed for the next launch ----
    __syncthreads();
    if (tid == 0) {
        if (T.overflow) atomicAdd(&a.acc[0], (unsigned long long)T.overflow);
        if (T.errflags) atomicOr(&a.acc[1], (unsigned long long)T.errflags);
        __threadfence();
        T.last = atomicAdd(&a.acc[2], 1ull) == (unsigned long long)gridDim.x - 1;
    }
    __syncthreads();
    if (T.last) {
        __threadfence();
        for (uint32_t i = tid; i < T.n; i += nthr) a.lookback[i] = 0ull;
        if (tid == 0) {
            if (T.n == 0) { a.totals[0] = 0ull; a.totals[1] = 0ull; }
            const unsigned long long t2 = atomicExch(&a.acc[0], 0ull), t3 = atomicExch(&a.acc[1], 0ull);
            a.totals[2] = t2;
            a.totals[3] = t3;
            atomicExch(&a.acc[2], 0ull);
            atomicExch(a.work_counter, 0u);
            if (a.host_totals) {
                // totals[0..1] came from the CTA that recorded the last ticket,
                // published before its count of finished CTAs
                a.host_totals[0] = __ldcg(&a.totals[0]);
                a.host_totals[1] = __ldcg(&a.totals[1]);
                a.host_totals[2] = t2;
                a.host_totals[3] = t3;
            }
        }
    }
}

// Planning pass of a batched build: the chunks the build kernel must take,
// in chunk order, into plan[1..n] and their number into plan[0].  A chunk
// whose depth bias alone decides every sample (bias_decides, the same test
// the build applies) needs neither noise nor mesh and is left out; a
// descriptor the build will flag as bad is listed.  Every CTA decides a slice
// of the batch (one descriptor per thread, so the reads are spread over the
// SMs) into one byte per chunk; the last CTA to finish compacts the bytes in
// chunk order, writes the records of the decided chunks before the first
// listed chunk (prefix 0; the build writes the others after the listed chunk
// before them) and re-arms the finish counter for the next launch.
constexpr int kPlanThreads = 256;
constexpr int kPlanPerThread = 16;  // chunks per thread in the compaction

__device__ __forceinline__ uint8_t* plan_kinds(uint32_t* plan, uint32_t n)
{
    return reinterpret_cast<uint8_t*>(plan) + plan_kinds_offset(n);
}

__global__ void __launch_bounds__(kPlanThreads) plan_kernel(const DevParams p, const BuildArgs a)
{
    // the build kernel may start its table setup now; it waits for this
    // grid's writes (griddepcontrol.wait) before reading the list
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    __shared__ uint32_t warp_count[kPlanThreads / 32];
    __shared__ uint32_t base;
    __shared__ int last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    uint8_t* kinds = plan_kinds(a.plan, a.n);
    const float B = fbm_bound(p);
    for (uint32_t i = blockIdx.x * kPlanThreads + tid; i < n; i += gridDim.x * kPlanThreads) {
        const uint32_t cells = __ldg(&a.chunks[i].cells);
        const int oz = __ldg(&a.chunks[i].pos[2]) * p.chunk_size;
        const bool ok = cells >= 1 && cells <= a.max_cells && cells <= UWW_MAX_CELLS;
        kinds[i] = ok ? (uint8_t)bias_decides_with(p, B, __fdiv_rn((float)p.chunk_size, (float)cells), (int)cells, oz)
                      : (uint8_t)0;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) last = atomicAdd(&a.plan[kPlanDone], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last CTA: compact, in chunk order
    if (tid == 0) base = 0;
    __syncthreads();
    constexpr uint32_t kTile = (uint32_t)kPlanThreads * kPlanPerThread;
    for (uint32_t t0 = 0; t0 < n; t0 += kTile) {
        const uint32_t i0 = t0 + (uint32_t)tid * kPlanPerThread;
        unsigned mine = 0;  // bit k: chunk i0 + k is listed
#pragma unroll
        for (int k = 0; k < kPlanPerThread; ++k)
            if (i0 + k < n && __ldcg(&kinds[i0 + k]) == 0) mine |= 1u << k;
        const uint32_t cnt = __popc(mine);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_count[warp] = incl;
        __syncthreads();
        uint32_t before = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kPlanThreads / 32; ++w) {
            const uint32_t v = warp_count[w];
            before += w < warp ? v : 0u;
            total += v;
        }
        uint32_t pos = kPlanList + base + before + incl - cnt;
        for (int k = 0; k < kPlanPerThread; ++k)
            if (mine & (1u << k)) a.plan[pos++] = i0 + k;
        __syncthreads();
        if (tid == 0) base += total;
        __syncthreads();
    }
    const uint32_t count = base;
    if (tid == 0) {
        a.plan[kPlanCount] = count;
        a.plan[kPlanDone] = 0u;  // re-armed for the next launch
    }
    const uint32_t first = count ? a.plan[kPlanList] : n;  // written by this CTA before the last barrier
    for (uint32_t j = tid; j < first; j += kPlanThreads) decided_record(a, j, __ldcg(&kinds[j]), 0ull, 0ull);
}

// ---------------------------------------------------------------------------
// Split build, for batches whose chunks (or slabs of them) all work in
// shared memory: the front half with the chunk-local pass 1, the records,
// and the rest of the emission, as separate kernels instead of one pipelined
// one.
//   split_plan_kernel (planned batches, and every batch with slabs): one
//     pass, one thread per chunk -- a chunk the depth bias decides gets its
//     counts word (zero, early-blank flag) at once (planned batches); the
//     others go to one of kPlanRanks work queues by cost rank
//     (bias_decides_with), the likely costliest first, a large chunk as its
//     slabs.
//   front_kernel: persistent, every thread a compute thread, one chunk per CTA
//     at a time from the queues -- noise, votes, classification and block scan
//     (chunk_front), then for a meshed chunk pass 1 from shared memory:
//     chunk-local indices and vertex positions into staging buffers (room
//     taken with one atomic per chunk), and the chunk's emission work as
//     units: blocks of its vertices, blocks of its indices.  Its counts go
//     to tinfo and to its tile's sum.  No look-back, no control warp, no
//     hand-offs, no ordering between CTAs.
//   emit_kernel, the front kernel's programmatic dependent: its first CTAs
//     write the records and totals, a tile of chunks each; then every CTA
//     takes units from a counter -- a vertex block's colours and normals
//     from its staged positions, an index block -- and, once the records
//     are written, stores them in place.  A chunk or slab the staging buffers
//     had no room for (the batch's output then exceeds the capacities) is
//     built again by one CTA and emitted in place.
// The same device functions as the pipelined build: the same bits.  The work
// order (queues, mesh list) varies from run to run; the outputs do not.

// ---------------------------------------------------------------------------
// Slabs of a large chunk (split build; layout and layer count: slab_layout).
// Slab s of a chunk of N cells per edge holds the cell layers x0 = s * K ..
// x1 - 1 and the sample planes x0 .. x1.  Its CTA's thread t owns a run of the
// slab's cell columns (x, y) -- N cells each, in the chunk's cell order -- so
// the slab's counts are one block scan.  A vertex is numbered by the cell that
// owns its edge; an edge on the slab's low x face is owned by a cell of the
// previous slab's last layer, which leaves per cell (y, z) its first vertex id
// and case in its seam, and the emission resolves those references from it.

struct SlabWs {
    float* rho;                   // (x - x0, y, z) samples of the slab's planes
    uint8_t* cases;               // per cell of the slab (active cells only)
    uint16_t* vbase;              // per active cell: first vertex id within the slab
    unsigned long long* masks;    // per sample column (x - x0, y): bits z with sample < iso
    uint32_t* alist;              // active cells in order: cell | first triangle << 16 (up to kSlabActCap)
};

__device__ __forceinline__ SlabWs slab_ws(uint8_t* base, int N)
{
    const SlabLayout L = slab_layout(N);
    SlabWs w;
    w.rho = reinterpret_cast<float*>(base + L.rho);
    w.cases = base + L.cases;
    w.vbase = reinterpret_cast<uint16_t*>(base + L.vbase);
    w.masks = reinterpret_cast<unsigned long long*>(base + L.masks);
    w.alist = reinterpret_cast<uint32_t*>(base + L.alist);
    return w;
}

// whether chunk `cells` is built as slabs (the planning kernel and the
// front kernel decide alike)
__device__ __forceinline__ bool slab_chunk(const BuildArgs& a, uint32_t cells)
{
    return a.pmax > 1 && cells > a.piece_cells && cells <= a.max_cells && cells <= (uint32_t)kSlabMaxCells;
}

// A cell column (x, y) of a slab: its four corner columns' masks and its
// active cells (bit z: the cell's corners are not all on one side)
struct SlabColumn {
    unsigned long long m00, m10, m01, m11, act, allin;
};

__device__ __forceinline__ SlabColumn slab_column(const unsigned long long* masks, int S, int xl, int y, int N)
{
    const int col = xl * S + y;
    SlabColumn c;
    c.m00 = masks[col];
    c.m10 = masks[col + S];
    c.m01 = masks[col + 1];
    c.m11 = masks[col + S + 1];
    const unsigned long long an = c.m00 & c.m10 & c.m01 & c.m11, no = ~(c.m00 | c.m10 | c.m01 | c.m11);
    c.allin = an & (an >> 1);
    const unsigned long long quiet = c.allin | (no & (no >> 1));
    c.act = ~quiet & ((1ull << N) - 1ull);
    return c;
}

// packed counts of an active cell: new vertices | indices << kIndShift | 1 active
__device__ __forceinline__ unsigned long long cell_counts(const SmemTables& T, int cs, unsigned own)
{
    return (unsigned long long)__popc(T.edges[cs] & own) | ((unsigned long long)(3 * T.ntri[cs]) << kIndShift) |
           (1ull << kActShift);
}

// Front half of slab s of chunk c into workspace W: the noise of its planes
// (fast build: the column form, which also leaves the columns' masks), the
// early-blank and solid votes, the classification from the masks, the block
// scan and each active cell's first vertex id.  The first time (first: the
// front kernel, not a rebuild) it also writes the last layer's ids and cases
// to the seam when a slab follows, and the slab's samples and cell cases when
// the batch asks for them.  Returns the slab's packed counts (every thread; 0
// when no cell is crossed); *any_inside: a sample is not above the iso level;
// *run: the thread's exclusive prefix.  Every thread (kSlabThreads) must call
// it.  GWS: W is in global memory (this CTA's scratch).
template <class O, bool GWS>
__device__ unsigned long long slab_front(const DevParams& p, const BuildArgs& a, SmemTables& T, const SlabWs W,
                                         uint8_t* ztab, const uww_chunk_desc d, uint32_t c, uint32_t s, int ncomp,
                                         bool first, int* any_inside_out, unsigned long long* run_out)
{
    const int tid = threadIdx.x;
    const int oriented = p.dedup_mode == UWW_DEDUP_ORIENTED;
    const int N = (int)d.cells, S = N + 1, K = slab_layers(N);
    const int x0 = (int)s * K, x1 = min(x0 + K, N), nl = x1 - x0, planes = nl + 1;
    const int ox = d.pos[0] * p.chunk_size, oy = d.pos[1] * p.chunk_size, oz = d.pos[2] * p.chunk_size;
    const float iso = p.iso_level;
    // a chunk the depth bias decides (met here when the batch is not planned:
    // its cases are written) needs no noise unless its samples are written
    const int decided = (first && !a.samples_out && !a.no_depth_shortcut) ? bias_decides(p, N, oz) : 0;
    int inside = decided == 2, outside = decided == 1;
    if (decided) {
    } else if constexpr (std::is_same<O, FastOps>::value) {
        // (columns of 25 and 49 samples accumulated in registers were no
        // faster, 49 much slower: the unrolled column outgrows the caches)
        const ZTable zt = ztable_at(ztab, S, p.octaves);
        // (a slab whose samples are not written may settle early as blank or
        // solid, after its first octaves, unless every noise is to be evaluated)
        const bool settle = first && !a.samples_out && !a.no_depth_shortcut && p.octaves >= kSettleMinOctaves;
        const int io =
            (!GWS && planes * S <= ncomp)
                ? sample_columns_fast_settle(p, T.perm, T.gp, zt, W.rho, N, ox, oy, oz, ncomp, W.masks, x0, planes,
                                             settle)
                : sample_columns_fast<GWS>(p, T.perm, T.gp, zt, W.rho, N, ox, oy, oz, ncomp, W.masks, x0, planes);
        inside = io & 1;
        outside = io >> 1;
    } else {
        const float sc = __fdiv_rn((float)p.chunk_size, (float)N);
        const int S2 = S * S;
        for (int idx = tid; idx < planes * S2; idx += ncomp) {
            const int xl = idx / S2, r = idx - xl * S2, y = r / S, z = r - y * S;
            const float wx = O::add(O::mul((float)(x0 + xl), sc), (float)ox);
            const float wy = O::add(O::mul((float)y, sc), (float)oy);
            const float wz = O::add(O::mul((float)z, sc), (float)oz);
            const float v = density<O, false>(p, T.perm, wx, wy, wz, nullptr);
            W.rho[idx] = v;
            inside |= !(v > iso);
            outside |= !(v < iso);
        }
    }
    const int any_inside = bar_or(kBarCompute, ncomp, inside);
    const int solid = bar_and(kBarCompute, ncomp, !outside);
    *any_inside_out = any_inside;
    *run_out = 0ull;
    // the samples and cell cases the batch asks for, within the capacities
    // the caller gave (the chunk's planes x0..x1 and cells of layers x0..x1-1)
    const bool want_cases = first && (p.outputs & UWW_OUT_CASES) != 0 && a.cases != nullptr;
    const bool cases_ok = want_cases && (unsigned long long)d.cell_offset + (unsigned long long)N * N * N <= a.case_capacity;
    const bool samples_ok = first && a.samples_out &&
                            (unsigned long long)d.sample_offset + (unsigned long long)S * S * S <= a.sample_capacity;
    if (tid == 0 && ((want_cases && !cases_ok) || (first && a.samples_out && !samples_ok)))
        atomicOr(&T.errflags, (uint32_t)kErrRange);
    if (samples_ok) {
        float* dst = a.samples_out + d.sample_offset + (size_t)x0 * S * S;
        for (int idx = tid; idx < planes * S * S; idx += ncomp) dst[idx] = W.rho[idx];
    }
    uint8_t* cases_out = cases_ok ? a.cases + d.cell_offset + (size_t)x0 * N * N : nullptr;
    if (!any_inside || solid) {
        if (cases_out)
            for (int k = tid; k < nl * N * N; k += ncomp) cases_out[k] = solid ? 255 : 0;
        return 0ull;
    }
    if constexpr (!std::is_same<O, FastOps>::value) {
        for (int col = tid; col < planes * S; col += ncomp) {
            unsigned long long m = 0ull;
            for (int z = 0; z < S; ++z) m |= (unsigned long long)(W.rho[col * S + z] < iso) << z;
            W.masks[col] = m;
        }
        bar_sync(kBarCompute, ncomp);
    }
    // ---- classify + count: the thread's run of cell columns ----
    const int ncol = nl * N, R = (ncol + ncomp - 1) / ncomp;
    const int q0 = min(tid * R, ncol), q1 = min(q0 + R, ncol);
    unsigned long long mine = 0ull;
    for (int q = q0; q < q1; ++q) {
        const int xl = q / N, y = q - xl * N, x = x0 + xl;
        const SlabColumn col = slab_column(W.masks, S, xl, y, N);
        const unsigned own_lo = (x == 0) | ((y == 0) << 1) | ((x == N - 1) << 3) | ((y == N - 1) << 4);
        if (cases_out)
            for (int z = 0; z < N; ++z)
                cases_out[q * N + z] = ((col.act >> z) & 1ull) ? (uint8_t)mask_case(col.m00, col.m10, col.m01, col.m11, z)
                                                               : ((col.allin >> z) & 1ull) ? 255 : 0;
        for (unsigned long long act = col.act; act; act &= act - 1ull) {
            const int z = __ffsll((long long)act) - 1;
            const int cs = mask_case(col.m00, col.m10, col.m01, col.m11, z);
            W.cases[q * N + z] = (uint8_t)cs;
            mine += cell_counts(T, cs, T.owned[oriented][own_lo | ((z == 0) << 2) | ((z == N - 1) << 5)]);
        }
    }
    unsigned long long total = 0ull;
    const unsigned long long run = block_exclusive_scan(mine, T, total, ncomp);
    *run_out = run;
    // ---- each active cell's first vertex id; the seam ----
    uint32_t* seam = first && (int)s + 1 < slab_count(N) ? a.seam + ((size_t)c * a.pmax + s) * a.seam_stride : nullptr;
    unsigned long long r = run;
    for (int q = q0; q < q1; ++q) {
        const int xl = q / N, y = q - xl * N, x = x0 + xl;
        const SlabColumn col = slab_column(W.masks, S, xl, y, N);
        const unsigned own_lo = (x == 0) | ((y == 0) << 1) | ((x == N - 1) << 3) | ((y == N - 1) << 4);
        for (unsigned long long act = col.act; act; act &= act - 1ull) {
            const int z = __ffsll((long long)act) - 1;
            const int cs = W.cases[q * N + z];
            W.vbase[q * N + z] = (uint16_t)(r & kField22);
            const uint32_t ar = (uint32_t)(r >> kActShift);
            if (ar < kSlabActCap)
                W.alist[ar] = (uint32_t)(q * N + z) | ((uint32_t)((r >> kIndShift) & kField22) / 3u) << 16;
            if (seam && x == x1 - 1) seam[y * N + z] = (uint32_t)(r & 0xffffu) | ((uint32_t)cs << 16);
            r += cell_counts(T, cs, T.owned[oriented][own_lo | ((z == 0) << 2) | ((z == N - 1) << 5)]);
        }
    }
    return total;
}

// A vertex of the previous slab, referenced from this one (staged index):
// kCrossRef | owner edge << 24 | the owner cell's y * N + z.
constexpr uint32_t kCrossRef = 0x80000000u;

// The chunk-local id of the vertex on edge oe of cell (x0 - 1, qy, qz) of the
// previous slab, from its seam (written by another kernel: read through L2);
// prev_base: that slab's first vertex in the chunk.
__device__ __forceinline__ uint32_t seam_vertex(const BuildArgs& a, const SmemTables& T, int oriented, int N,
                                                const uint32_t* seam_prev, int x0, int qy, int qz, int oe,
                                                uint32_t prev_base)
{
    const uint32_t w = __ldcg(seam_prev + qy * N + qz);
    const unsigned oown = T.owned[oriented][boundary_flags(x0 - 1, qy, qz, N)];
    return prev_base + (w & 0xffffu) + __popc(oown & __ldg(&UWW_EDGE_BEFORE[(w >> 16) & 255u][oe]));
}

// Pass 1 of a slab, from workspace W (this thread's run of cell columns,
// prefix `run`): per active cell its triangles' indices and the positions of
// the vertices it creates.  Staged (!FINAL): slab-local vertex ids (a vertex of
// the previous slab as a kCrossRef word) at eo.inds + ioff, positions (with the
// owner's corner b) at eo.pos + voff.  FINAL: chunk-local ids (vbase0: the
// slab's first vertex in the chunk, prev_base: the previous slab's) into the
// outputs at ioff and voff, colour slot 0 carrying corner b when pass 2
// follows (carry).
template <class O, bool FINAL>
__device__ void slab_emit(const DevParams& p, const BuildArgs& a, const SmemTables& T, const SlabWs W,
                          const uww_chunk_desc d, uint32_t c, uint32_t s, unsigned long long run,
                          unsigned long long total, int ncomp, const EmitOut& eo, uint32_t voff, uint32_t ioff,
                          uint32_t vbase0, uint32_t prev_base, bool carry)
{
    const int tid = threadIdx.x;
    const int oriented = p.dedup_mode == UWW_DEDUP_ORIENTED;
    const int N = (int)d.cells, S = N + 1, K = slab_layers(N);
    const int x0 = (int)s * K, x1 = min(x0 + K, N), nl = x1 - x0;
    const int ox = d.pos[0] * p.chunk_size, oy = d.pos[1] * p.chunk_size, oz = d.pos[2] * p.chunk_size;
    const float sc = __fdiv_rn((float)p.chunk_size, (float)N);
    const uint32_t* seam_prev = s > 0 ? a.seam + ((size_t)c * a.pmax + s - 1) * a.seam_stride : nullptr;
    // active cell (xl, y, z) of the slab (index cell, case cs, first vertex
    // vb and first index position ir within the slab): its triangles
    auto emit_cell = [&](int xl, int y, int z, int cell, int cs, uint32_t vb, uint32_t ir) {
        const int x = x0 + xl;
        const unsigned own = T.owned[oriented][boundary_flags(x, y, z, N)];
        const int nt = T.ntri[cs];
        const int8_t* row = T.tri[cs];
        const unsigned fr = T.first_ref[cs];
        const uint16_t* before = UWW_EDGE_BEFORE[cs];
        const int lo = (x == 0) | ((y == 0) << 1) | ((z == 0) << 2);
        for (int i = 0; i < 3 * nt; ++i) {
            const int e = row[i];
            uint32_t id;
            if ((own >> e) & 1u) {
                // the cell numbers its owned edges' vertices in first-reference order
                id = vb + __popc(own & __ldg(before + e));
                if ((fr >> i) & 1u) {
                    const EdgeVertex ev = edge_vertex<O>(p, T, W.rho, S, x, y, z, e, sc, ox, oy, oz, x0);
                    if (eo.edge_ids) eo.edge_ids[voff + id] = ev.edge_id;
                    if (FINAL) {
                        float2* v2 = reinterpret_cast<float2*>(eo.verts + voff + id);
                        v2[0] = make_float2(ev.x, ev.y);
                        v2[1] = make_float2(ev.z, carry ? (float)ev.cb : 0.f);
                        v2[2] = make_float2(0.f, 0.f);
                    } else {
                        eo.pos[voff + id] = make_float4(ev.x, ev.y, ev.z, (float)ev.cb);
                    }
                }
                if (FINAL) id += vbase0;
            } else {
                // the owner: the first cell in stream order holding this edge
                const int ow = T.owner[oriented][lo][e];
                const int qx = x - ((ow >> 4) & 1), qy = y - ((ow >> 5) & 1), qz = z - ((ow >> 6) & 1);
                const int oe = ow & 15;
                if (qx < x0) {
                    id = FINAL ? seam_vertex(a, T, oriented, N, seam_prev, x0, qy, qz, oe, prev_base)
                               : kCrossRef | ((uint32_t)oe << 24) | (uint32_t)(qy * N + qz);
                } else {
                    const int oc = ((qx - x0) * N + qy) * N + qz;
                    const unsigned oown = T.owned[oriented][boundary_flags(qx, qy, qz, N)];
                    id = (uint32_t)W.vbase[oc] + __popc(oown & __ldg(&UWW_EDGE_BEFORE[W.cases[oc]][oe]));
                    if (FINAL) id += vbase0;
                }
            }
            eo.inds[ioff + ir + i] = id;
        }
    };
    const uint32_t nA = (uint32_t)(total >> kActShift);
    if (nA <= kSlabActCap) {
        // a thread per active cell, from the list the scan filled
        for (uint32_t k = tid; k < nA; k += ncomp) {
            const uint32_t en = W.alist[k];
            const int cell = (int)(en & 0xffffu), q = cell / N, z = cell - q * N, xl = q / N;
            emit_cell(xl, q - xl * N, z, cell, W.cases[cell], W.vbase[cell], 3u * (en >> 16));
        }
        return;
    }
    // (more active cells than the list holds) each thread its run of columns
    const int ncol = nl * N, R = (ncol + ncomp - 1) / ncomp;
    const int q0 = min(tid * R, ncol), q1 = min(q0 + R, ncol);
    unsigned long long r = run;
    for (int q = q0; q < q1; ++q) {
        const int xl = q / N, y = q - xl * N;
        const SlabColumn col = slab_column(W.masks, S, xl, y, N);
        for (unsigned long long act = col.act; act; act &= act - 1ull) {
            const int z = __ffsll((long long)act) - 1;
            const int cs = W.cases[q * N + z];
            emit_cell(xl, y, z, q * N + z, cs, (uint32_t)(r & kField22), (uint32_t)((r >> kIndShift) & kField22));
            r += cell_counts(T, cs, T.owned[oriented][boundary_flags(x0 + xl, y, z, N)]);
        }
    }
}

// counts word of a chunk the depth bias decides (kind 1: every sample above
// the iso level -- early blank; 2: every sample below it)
__device__ __forceinline__ unsigned long long decided_info(int kind) { return kind == 1 ? kInfoEarlyBlank : 0ull; }

__global__ void __launch_bounds__(kPlanThreads) split_plan_kernel(const DevParams p, const BuildArgs a)
{
    // the front kernel may start its table setup now; it waits for this
    // grid's writes (griddepcontrol.wait) before taking work
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const uint32_t n = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    const float B = fbm_bound(p);
    for (uint32_t i = blockIdx.x * kPlanThreads + threadIdx.x; i < n; i += gridDim.x * kPlanThreads) {
        const uint32_t cells = __ldg(&a.chunks[i].cells);
        const int oz = __ldg(&a.chunks[i].pos[2]) * p.chunk_size;
        const bool ok = cells >= 1 && cells <= a.max_cells && cells <= UWW_MAX_CELLS;
        int rank = 0;
        const int kind = (ok && a.split_decide)
                             ? bias_decides_with(p, B, __fdiv_rn((float)p.chunk_size, (float)cells), (int)cells, oz, &rank)
                             : 0;
        if (kind) {
            a.tinfo[i] = decided_info(kind);
        } else if (ok && slab_chunk(a, cells)) {
            // a chunk built as slabs: every slab queued first, as the
            // largest pieces of work (those of chunks above 32 cells, the
            // longest, in queue 0; the rest in queue 1); its counts word
            // starts at zero counts and early blank, and each slab adds its
            // counts and clears the flag when one of its samples is not above
            // the iso level
            const uint32_t np = (uint32_t)slab_count((int)cells), qcap = a.n * a.pmax;
            const uint32_t q = cells > 32 ? 0u : 1u;
            a.tinfo[i] = kInfoEarlyBlank;
            const uint32_t pos = atomicAdd(&a.split_ctr[kCtrQueued + q], np);
            for (uint32_t sl = 0; sl < np; ++sl)
                if (pos + sl < qcap) a.split_queue[(size_t)q * qcap + pos + sl] = i | (sl << kPieceShift);
        } else {
            // (the counters are zero at launch, so pos < n * pmax; checked all the same)
            const uint32_t qcap = a.n * a.pmax;
            // with slabs, whole chunks queue after them (queues 2..)
            if (a.pmax > 1) rank = min(rank + 2, kPlanRanks - 1);
            const uint32_t pos = atomicAdd(&a.split_ctr[kCtrQueued + rank], 1u);
            if (pos < qcap) a.split_queue[(size_t)rank * qcap + pos] = i;
        }
    }
}

// The split build's next piece of work for this CTA (thread 0): a chunk from
// the first queue with work left (planned), else the next chunk in order;
// kNoChunk when there is none.
constexpr uint32_t kNoChunk = 0xffffffffu;
__device__ __forceinline__ uint32_t split_take(const BuildArgs& a, uint32_t nchunks, uint32_t& rank)
{
    if (!a.split_planned) {
        const uint32_t k = atomicAdd(&a.split_ctr[kCtrTaken], 1u);
        return k < nchunks ? k : kNoChunk;
    }
    const uint32_t qcap = a.n * a.pmax;
    while (rank < (uint32_t)kPlanRanks) {
        const uint32_t k = atomicAdd(&a.split_ctr[kCtrTaken + rank], 1u);
        if (k < min(__ldcg(&a.split_ctr[kCtrQueued + rank]), qcap)) return __ldcg(&a.split_queue[(size_t)rank * qcap + k]);
        ++rank;
    }
    return kNoChunk;
}

// The front kernel's work on slab s of chunk c: its front half in the shared
// workspace, its counts to the chunk's counts word, its place's counts and the
// chunk's tile sum, then (meshed) its staged pass 1 and its emission units --
// or, when the staging buffers have no room, one unit for the emission kernel
// to build the slab again and emit it in place.
template <class O>
__device__ void front_slab(const DevParams& p, const BuildArgs& a, SmemTables& T, uint8_t* dyn_smem,
                           const uww_chunk_desc d, uint32_t c, uint32_t sl, unsigned long long& stage,
                           uint32_t& unit_a, uint32_t& unit_b)
{
    const int tid = threadIdx.x, nthr = blockDim.x;
    const uint32_t place = c * a.pmax + sl;
    const SlabWs W = slab_ws(dyn_smem, (int)d.cells);
    int any_inside = 0;
    unsigned long long run = 0ull;
    const unsigned long long tot = slab_front<O, false>(p, a, T, W, dyn_smem + a.ztable_offset, d, c, sl, nthr, true,
                                                        &any_inside, &run);
    const uint32_t nV = (uint32_t)(tot & kField22), nI = (uint32_t)((tot >> kIndShift) & kField22);
    const uint32_t vb = (nV + kVertexBlock - 1) / kVertexBlock, ib = (nI + kIndexBlock - 1) / kIndexBlock;
    if (tid == 0) {
        if (tot) atomicAdd(&a.tinfo[c], tot);
        if (any_inside) atomicAnd(&a.tinfo[c], ~kInfoEarlyBlank);
        a.pinfo[place] = (unsigned long long)nV | ((unsigned long long)nI << 32);
        if (nV | nI) atomicAdd(&a.tile_sum[c / kTileChunks], (unsigned long long)nV | ((unsigned long long)nI << 32));
        if (nI) {
            const unsigned long long at =
                atomicAdd(a.stage_ctr, (unsigned long long)nV | ((unsigned long long)nI << 32));
            const unsigned long long sv = at & 0xffffffffull, si = at >> 32;
            const bool room = sv + nV <= a.stage_vcap && si + nI <= a.stage_icap;
            stage = room ? at : kUnstaged;
            a.stage_at[place] = stage;
            unit_a = atomicAdd(&a.split_ctr[kCtrUnitsA], room ? vb : 1u);
            unit_b = room ? atomicAdd(&a.split_ctr[kCtrUnitsB], ib) : 0u;
        }
    }
    __syncthreads();
    if (!nI) return;
    const unsigned long long st = stage;
    if (st != kUnstaged) {
        const EmitOut eo{nullptr, a.stage_inds, a.edge_ids ? a.stage_eids : nullptr, a.stage_pos};
        slab_emit<O, false>(p, a, T, W, d, c, sl, run, tot, nthr, eo, (uint32_t)st, (uint32_t)(st >> 32), 0u, 0u,
                            true);
        for (uint32_t k = tid; k < vb; k += nthr)
            if (unit_a + k < a.unit_cap) a.units[unit_a + k] = unit_entry(c, k | (sl << 16), kUnitVerts | kUnitSlab);
        for (uint32_t k = tid; k < ib; k += nthr)
            if (unit_b + k < a.unit_cap)
                a.units[a.unit_cap - 1 - (unit_b + k)] = unit_entry(c, k | (sl << 16), kUnitInds | kUnitSlab);
    } else if (tid == 0 && unit_a < a.unit_cap) {
        a.units[unit_a] = unit_entry(c, sl << 16, kUnitChunk | kUnitSlab);
    }
}

template <class O, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) front_kernel(const DevParams p, const BuildArgs a)
{
    extern __shared__ __align__(16) uint8_t dyn_smem[];
    __shared__ SmemTables T;
    __shared__ uint32_t rank, unit_a, unit_b;
    __shared__ unsigned long long stage;
    const int tid = threadIdx.x, nthr = blockDim.x;
    load_tables_image(p, a, T, tid, nthr);
    // the planning kernel's queues (this kernel is its programmatic dependent)
    if (a.split_planned) asm volatile("griddepcontrol.wait;" ::: "memory");
    // the records kernel, launched after this one as its programmatic
    // dependent (and the emission kernel after it), may take SMs as this
    // kernel's CTAs finish; each waits for the kernel before it
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (tid == 0) {
        T.errflags = 0;
        T.nchunks = a.n_dev ? min(*a.n_dev, a.n) : a.n;
        rank = 0;
        // the records kernel adds the chunks that do not fit
        if (blockIdx.x == 0) a.totals[2] = 0ull;
    }
    __syncthreads();
    for (;;) {
        if (tid == 0) {
            const uint32_t e = split_take(a, T.nchunks, rank);
            // a queue entry of a batch with slabs: chunk | slab << kPieceShift
            const uint32_t c = (e == kNoChunk || a.pmax == 1) ? e : (e & ((1u << kPieceShift) - 1u));
            T.tk[0].chunk = c;
            T.tk[0].ticket = (e == kNoChunk || a.pmax == 1) ? 0u : e >> kPieceShift;
            if (c != kNoChunk) T.tk[0].desc = a.chunks[c];
        }
        __syncthreads();
        const uint32_t c = T.tk[0].chunk;
        if (c == kNoChunk) break;
        if constexpr (MAXT == kSlabThreads && MINB == 2) {
            if (slab_chunk(a, T.tk[0].desc.cells)) {
                front_slab<O>(p, a, T, dyn_smem, T.tk[0].desc, c, T.tk[0].ticket, stage, unit_a, unit_b);
                __syncthreads();  // the workspace and the staged ticket are reused
                continue;
            }
        }
        const uint32_t place = c * a.pmax;
        chunk_front<O, false>(p, a, T, dyn_smem, T.tk[0].desc, c, c, 0, nthr);
        __syncthreads();
        const ChunkInfo ci = T.ci[0];
        const uint32_t nV = (uint32_t)(ci.total & kField22), nI = (uint32_t)((ci.total >> kIndShift) & kField22);
        // the chunk's emission work: blocks of kVertexBlock vertices (colour,
        // normal; list A) and of kIndexBlock indices (list B) when its pass 1
        // is staged, else the whole chunk, built again (list A)
        const uint32_t vb = (nV + kVertexBlock - 1) / kVertexBlock, ib = (nI + kIndexBlock - 1) / kIndexBlock;
        if (tid == 0) {
            a.tinfo[c] = ci.total | ((ci.flags & UWW_CHUNK_EARLY_BLANK) ? kInfoEarlyBlank : 0ull);
            if (nV | nI) atomicAdd(&a.tile_sum[c / kTileChunks], (unsigned long long)nV | ((unsigned long long)nI << 32));
            if (nI) {
                // room in the staging buffers (first come, first served; they
                // hold the batch whenever its output fits its capacities)
                const unsigned long long at =
                    atomicAdd(a.stage_ctr, (unsigned long long)nV | ((unsigned long long)nI << 32));
                const unsigned long long sv = at & 0xffffffffull, si = at >> 32;
                const bool room = sv + nV <= a.stage_vcap && si + nI <= a.stage_icap;
                stage = room ? at : kUnstaged;
                a.stage_at[place] = stage;
                unit_a = atomicAdd(&a.split_ctr[kCtrUnitsA], room ? vb : 1u);
                unit_b = room ? atomicAdd(&a.split_ctr[kCtrUnitsB], ib) : 0u;
            }
        }
        __syncthreads();
        if (nI) {
            const unsigned long long st = stage;
            if (st != kUnstaged) {
                // pass 1 from the shared workspace: chunk-local indices and
                // vertex positions (with the owner's corner b) into staging
                const int N = ci.N;
                const Workspace W = workspace(a, dyn_smem, 0, N);
                const uint32_t sv = (uint32_t)st, si = (uint32_t)(st >> 32);
                const uint32_t nT = nI / 3u, nA = (uint32_t)(ci.total >> kActShift);
                const bool direct = direct_triangles(W, N, ci.total);
                const float s = __fdiv_rn((float)p.chunk_size, (float)N);
                const EmitOut eo{nullptr, a.stage_inds, a.edge_ids ? a.stage_eids : nullptr, a.stage_pos};
                for (uint32_t t = tid; t < nT; t += nthr)
                    emit_triangle<O>(p, eo, T, W, N, nA, direct, t, sv, si, ci.ox, ci.oy, ci.oz, s, true);
                for (uint32_t k = tid; k < vb; k += nthr)
                    if (unit_a + k < a.unit_cap) a.units[unit_a + k] = unit_entry(c, k, kUnitVerts);
                for (uint32_t k = tid; k < ib; k += nthr)
                    if (unit_b + k < a.unit_cap) a.units[a.unit_cap - 1 - (unit_b + k)] = unit_entry(c, k, kUnitInds);
            } else if (tid == 0 && unit_a < a.unit_cap) {
                // no room: one unit, for the emission kernel to build the
                // chunk again and emit it in place
                a.units[unit_a] = unit_entry(c, 0, kUnitChunk);
            }
        }
        __syncthreads();  // the workspace and the staged ticket are reused
    }
    if (tid == 0 && T.errflags) atomicOr(&a.acc[1], (unsigned long long)T.errflags);
}

// Acquire load at gpu scope: the emission kernel's CTAs learn through it
// that the records of every tile are written.
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 of a CTA: wait (bounded, backing off) until cond() holds; on
// timeout raise the error flag and return false.
template <class F>
__device__ __forceinline__ bool wait_until(const BuildArgs& a, F cond)
{
    const long long t0 = clock64();
    unsigned ns = 32;
    while (!cond()) {
        if (clock64() - t0 > a.spin_limit_cycles) {
            atomicOr(&a.acc[1], (unsigned long long)kErrTimeout);
            return false;
        }
        __nanosleep(ns);
        ns = min(2u * ns, 256u);
    }
    return true;
}

// a chunk's record, through L2 (written by another CTA of the emission kernel)
__device__ __forceinline__ uww_chunk_record load_record(const uww_chunk_record* r)
{
    uww_chunk_record rec;
    const uint4* r4 = reinterpret_cast<const uint4*>(r);
    *reinterpret_cast<uint4*>(&rec) = __ldcg(r4);
    *(reinterpret_cast<uint4*>(&rec) + 1) = __ldcg(r4 + 1);
    return rec;
}

// The emission kernel's work on a slab the staging buffers had no room for:
// its front half again in this CTA's global scratch (the seam is the front
// kernel's), then pass 1 into the outputs at voff (its first vertex, chunk
// id vbase0; the previous slab's first vertex prev_base) and ioff, and pass 2
// over its nv vertices.  Kept out of line: the emission's other units do not
// pay for its registers.
template <class O>
__device__ __noinline__ void emit_slab_again(const DevParams& p, const BuildArgs& a, SmemTables& T, uint8_t* dyn_smem,
                                             uint32_t c, uint32_t sl, uint32_t voff, uint32_t ioff, uint32_t vbase0,
                                             uint32_t prev_base, uint32_t nv)
{
    const int tid = threadIdx.x, nthr = blockDim.x;
    const bool want_color = (p.outputs & UWW_OUT_COLOR) != 0;
    const bool want_normals = (p.outputs & UWW_OUT_NORMALS) != 0 && a.normals != nullptr;
    const uww_chunk_desc d = a.chunks[c];
    const SlabWs W = slab_ws(a.scratch + (size_t)blockIdx.x * a.scratch_slot_bytes, (int)d.cells);
    int any_inside = 0;
    unsigned long long run = 0ull;
    const unsigned long long total = slab_front<O, true>(p, a, T, W, dyn_smem, d, c, sl, nthr, false, &any_inside, &run);
    __syncthreads();
    const EmitOut eo{a.verts, a.inds, a.edge_ids, nullptr};
    slab_emit<O, true>(p, a, T, W, d, c, sl, run, total, nthr, eo, voff, ioff, vbase0, prev_base,
                       want_color || want_normals);
    if (want_color || want_normals) {
        __syncthreads();  // the slab's vertex positions, written by this CTA
        for (uint32_t v = tid; v < nv; v += nthr)
            finish_vertex<O>(p, T.perm, T.gp, a.verts, a.normals, voff + v, want_color, want_normals);
    }
}

// The emission kernel's work on a whole chunk the staging buffers had no
// room for: its front half again in this CTA's global scratch slot (shared
// memory as rebuild_layout says; its cases and samples are the front
// kernel's), then pass 1 into the outputs at its record's offsets and pass 2.
// Kept out of line, like emit_slab_again.
template <class O>
__device__ __noinline__ void emit_chunk_again(const DevParams& p, const BuildArgs& a, SmemTables& T, uint8_t* dyn_smem,
                                              uint32_t c, const uww_chunk_record rec)
{
    const int tid = threadIdx.x, nthr = blockDim.x;
    const bool want_color = (p.outputs & UWW_OUT_COLOR) != 0;
    const bool want_normals = (p.outputs & UWW_OUT_NORMALS) != 0 && a.normals != nullptr;
    BuildArgs b = a;
    b.cases = nullptr;
    b.samples_out = nullptr;
    // every chunk in the scratch slot: the masks at the start of the dynamic
    // shared memory, the z tables after them
    size_t zt = 0;
    rebuild_layout((int)a.smem_cells, (int)p.octaves, std::is_same<O, FastOps>::value, &zt);
    b.smem_cells = 0;
    b.slots_per_cta = 1;
    b.smem_buf_bytes = zt;
    b.ztable_offset = zt;
    b.mask_offset = 0;
    const uww_chunk_desc d = a.chunks[c];
    chunk_front<O, false>(p, b, T, dyn_smem, d, c, c, 0, nthr);
    __syncthreads();
    const int N = (int)d.cells;
    const Workspace W = workspace(b, dyn_smem, 0, N);
    const bool direct = direct_triangles(W, N, T.ci[0].total);
    const float s = __fdiv_rn((float)p.chunk_size, (float)N);
    const EmitOut eo{a.verts, a.inds, a.edge_ids, nullptr};
    for (uint32_t tr = tid; tr < rec.num_inds / 3u; tr += nthr)
        emit_triangle<O>(p, eo, T, W, N, rec.num_active_cells, direct, tr, rec.vert_offset, rec.ind_offset,
                         d.pos[0] * p.chunk_size, d.pos[1] * p.chunk_size, d.pos[2] * p.chunk_size, s,
                         want_color || want_normals);
    if (want_color || want_normals) {
        __syncthreads();  // the chunk's vertex positions, written by this CTA
        for (uint32_t v = tid; v < rec.num_verts; v += nthr)
            finish_vertex<O>(p, T.perm, T.gp, a.verts, a.normals, rec.vert_offset + v, want_color, want_normals);
    }
}

template <class O>
__global__ void __launch_bounds__(256, 4) emit_kernel(const DevParams p, const BuildArgs a)
{
    // a chunk built again (chunks without staging room) or a gathered vertex block
    extern __shared__ __align__(16) uint8_t dyn_smem[];
    __shared__ SmemTables T;
    __shared__ int last;
    __shared__ uint32_t next_ticket;
    __shared__ int rec_wait;
    const int tid = threadIdx.x, nthr = blockDim.x;
    load_tables_image(p, a, T, tid, nthr);
    // launched as a programmatic dependent of the front kernel: what it
    // wrote is read after this, through L2
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t nchunks = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    const uint32_t ntiles = (nchunks + kTileChunks - 1) / kTileChunks;
    const uint32_t na = min(__ldcg(&a.split_ctr[kCtrUnitsA]), a.unit_cap);
    const uint32_t nb = min(__ldcg(&a.split_ctr[kCtrUnitsB]), a.unit_cap - na);
    const uint32_t nunits = na + nb;
    const bool want_color = (p.outputs & UWW_OUT_COLOR) != 0;
    const bool want_normals = (p.outputs & UWW_OUT_NORMALS) != 0 && a.normals != nullptr;
    // ---- the records: warp 0 of the first CTAs, one tile of kTileChunks
    // (32) chunks each (a lane per chunk), so that the record warps spread
    // over the SMs -- the tiles before it summed from the tile sums (all
    // loads in flight together), then a warp scan; no CTA barrier ----
    {
        const int lane = tid & 31, warp = tid >> 5;
        uint32_t tiles = 0;
        unsigned long long over = 0;
        if (warp == 0)
            for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++tiles) {
                const uint32_t j = tile * kTileChunks + lane;
                const unsigned long long w = j < nchunks ? __ldcg(&a.tinfo[j]) : 0ull;
                unsigned long long pv = 0ull, pi = 0ull;
                for (uint32_t k0 = 0; k0 < tile; k0 += 8 * 32) {
                    unsigned long long sm[8];
#pragma unroll
                    for (int r = 0; r < 8; ++r) {
                        const uint32_t k = k0 + (uint32_t)r * 32u + lane;
                        sm[r] = k < tile ? __ldcg(&a.tile_sum[k]) : 0ull;
                    }
#pragma unroll
                    for (int r = 0; r < 8; ++r) {
                        pv += sm[r] & 0xffffffffull;
                        pi += sm[r] >> 32;
                    }
                }
                const uint32_t nV = (uint32_t)(w & kField22), nI = (uint32_t)((w >> kIndShift) & kField22);
                unsigned long long ev = nV, ei = nI;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    pv += __shfl_xor_sync(0xffffffffu, pv, o);
                    pi += __shfl_xor_sync(0xffffffffu, pi, o);
                }
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned long long xv = __shfl_up_sync(0xffffffffu, ev, o),
                                             xi = __shfl_up_sync(0xffffffffu, ei, o);
                    if (lane >= o) { ev += xv; ei += xi; }
                }
                ev += pv - nV;  // exclusive prefix of chunk j
                ei += pi - nI;
                if (j < nchunks) {
                    const bool fits = ev + nV <= a.vert_capacity && ei + nI <= a.ind_capacity;
                    uww_chunk_record rec;
                    rec.num_verts = nV;
                    rec.num_inds = nI;
                    rec.vert_offset = rec_off32(ev);
                    rec.ind_offset = rec_off32(ei);
                    rec.flags = ((w & kInfoEarlyBlank) ? UWW_CHUNK_EARLY_BLANK : 0u) |
                                (nI ? UWW_CHUNK_HAS_MESH : 0u) | (fits ? 0u : UWW_CHUNK_OVERFLOW);
                    rec.num_active_cells = (uint32_t)((w >> kActShift) & 0x3ffffull);
                    rec.reserved[0] = rec.reserved[1] = 0;
                    a.records[j] = rec;
                    over += fits ? 0u : 1u;
                }
            }
        if (tiles) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) over += __shfl_xor_sync(0xffffffffu, over, o);
            // published: this warp's tiles, for every CTA's units
            __threadfence();
            __syncwarp();
            if (lane == 0) {
                if (over) atomicAdd(&a.totals[2], over);
                // (failure injection: tile 0, this warp's first, never announced)
                const uint32_t told = tiles - ((a.withhold_records && blockIdx.x == 0) ? 1u : 0u);
                if (told) atomicAdd(&a.split_ctr[kCtrRecDone], told);
            }
        }
        if (blockIdx.x == 0 && warp == 1) {
            // the totals, from every tile's sum
            unsigned long long v = 0ull, i = 0ull;
            for (uint32_t k = lane; k < ntiles; k += 32) {
                const unsigned long long sm = __ldcg(&a.tile_sum[k]);
                v += sm & 0xffffffffull;
                i += sm >> 32;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                v += __shfl_xor_sync(0xffffffffu, v, o);
                i += __shfl_xor_sync(0xffffffffu, i, o);
            }
            if (lane == 0) {
                a.totals[0] = v;
                a.totals[1] = i;
            }
        }
    }
    // the records every unit needs are waited for only once its own work
    // is done, just before its first store (a CTA's first unit overlaps
    // the records' writing); if the wait runs out, the CTA stores nothing
    bool recs = false, recs_ok = false;
    auto await_records = [&]() -> bool {
        if (!recs) {
            if (tid == 0)
                rec_wait = wait_until(a, [&]() { return ld_acquire_u32(&a.split_ctr[kCtrRecDone]) >= ntiles; }) ? 1 : 0;
            __syncthreads();
            recs_ok = rec_wait != 0;
            recs = true;
        }
        return recs_ok;
    };
    // ticket t: list A (vertex blocks, whole chunks) first, then list B
    // (index blocks); tickets below gridDim.x are static, the rest counted
    uint32_t t = blockIdx.x;
    while (t < nunits) {
        const unsigned long long ent = t < na ? __ldcg(&a.units[t]) : __ldcg(&a.units[a.unit_cap - 1 - (t - na)]);
        const uint32_t c = (uint32_t)ent, kind = (uint32_t)(ent >> 60) & 7u;
        const bool slab = (ent >> 63) != 0ull;
        uint32_t part = (uint32_t)(ent >> 32) & 0x0fffffffu, sl = 0;
        if (slab) {
            sl = part >> 16;
            part &= 0xffffu;
        }
        const uint32_t place = c * a.pmax + sl;
        const unsigned long long w = __ldcg(&a.tinfo[c]);
        // a slab's own counts, where it starts in its chunk (bv, bi) and
        // where the slab before it starts (pv): sums over the slabs before
        uint32_t cnV = (uint32_t)(w & kField22), cnI = (uint32_t)((w >> kIndShift) & kField22);
        uint32_t bv = 0, bi = 0, pv = 0;
        if (slab) {
            const unsigned long long* pi = a.pinfo + (size_t)c * a.pmax;
            for (uint32_t j = 0; j < sl; ++j) {
                const unsigned long long x = __ldcg(pi + j);
                pv = bv;
                bv += (uint32_t)x;
                bi += (uint32_t)(x >> 32);
            }
            const unsigned long long own = __ldcg(pi + sl);
            cnV = (uint32_t)own;
            cnI = (uint32_t)(own >> 32);
        }
        __syncthreads();  // every thread has read the previous next_ticket
        if (tid == 0) next_ticket = gridDim.x + atomicAdd(&a.split_ctr[kCtrUnitsTaken], 1u);
        {
            if (kind == kUnitVerts) {
                // colour and normal of a block of the chunk's vertices, from
                // their staged positions, gathered in shared memory; then (the
                // record known) the block's vertices and normals to their
                // place as consecutive 4-byte words, whole sectors per warp
                // (the outputs may be page-locked host memory)
                const uint32_t v0 = part * kVertexBlock, v = v0 + tid;
                const uint32_t nv = cnV > v0 ? min(kVertexBlock, cnV - v0) : 0u;
                float* sw = reinterpret_cast<float*>(dyn_smem);  // 6 words a vertex, then 3 a normal
                if (tid < (int)nv) {
                    const uint32_t sv = (uint32_t)__ldcg(&a.stage_at[place]);
                    const float4 q = __ldcg(a.stage_pos + sv + v);
                    float2 out[3];
                    float g[3];
                    vertex_values<O>(p, T.perm, T.gp, make_float2(q.x, q.y), make_float2(q.z, q.w), want_color,
                                     want_normals, out, g);
                    float* o = sw + 6 * tid;
                    o[0] = out[0].x; o[1] = out[0].y; o[2] = out[1].x; o[3] = out[1].y; o[4] = out[2].x; o[5] = out[2].y;
                    float* nn = sw + 6 * kVertexBlock + 3 * tid;
                    nn[0] = g[0]; nn[1] = g[1]; nn[2] = g[2];
                }
                const bool ok = await_records();
                __syncthreads();  // the block is gathered
                const uww_chunk_record rec = load_record(&a.records[c]);
                if (ok && !(rec.flags & UWW_CHUNK_OVERFLOW)) {
                    if (a.edge_ids && tid < (int)nv)
                        a.edge_ids[rec.vert_offset + bv + v] =
                            __ldcg(a.stage_eids + (uint32_t)__ldcg(&a.stage_at[place]) + v);
                    float* dv = reinterpret_cast<float*>(a.verts + rec.vert_offset + bv + v0);
                    for (uint32_t k = tid; k < 6 * nv; k += nthr) dv[k] = sw[k];
                    if (want_normals) {
                        float* dn = a.normals + 3 * (size_t)(rec.vert_offset + bv + v0);
                        for (uint32_t k = tid; k < 3 * nv; k += nthr) dn[k] = sw[6 * kVertexBlock + k];
                    }
                }
            } else if (kind == kUnitInds) {
                // a block of the chunk's indices (loaded), then to their place
                const uint32_t si = (uint32_t)(__ldcg(&a.stage_at[place]) >> 32);
                const uint32_t k0 = part * kIndexBlock, k1 = min(k0 + kIndexBlock, cnI);
                const uint32_t* src = a.stage_inds + si;
                uint32_t iw[kIndexBlock / 256];
#pragma unroll
                for (int r = 0; r < (int)(kIndexBlock / 256); ++r) {
                    const uint32_t k = k0 + (uint32_t)r * 256u + tid;
                    iw[r] = k < k1 ? __ldcg(src + k) : 0u;
                }
                if (slab) {
                    // slab-local ids to chunk-local; a vertex of the previous
                    // slab from that slab's seam
                    const int N = (int)__ldg(&a.chunks[c].cells);
                    const int oriented = p.dedup_mode == UWW_DEDUP_ORIENTED;
                    const int x0 = (int)sl * slab_layers(N);
                    const uint32_t* seam_prev =
                        sl > 0 ? a.seam + ((size_t)c * a.pmax + sl - 1) * a.seam_stride : nullptr;
#pragma unroll
                    for (int r = 0; r < (int)(kIndexBlock / 256); ++r) {
                        const uint32_t v = iw[r];
                        if ((v & kCrossRef) && seam_prev) {
                            const int qyz = (int)(v & 0xffffffu) % (N * N);
                            iw[r] = seam_vertex(a, T, oriented, N, seam_prev, x0, qyz / N, qyz % N,
                                                (int)((v >> 24) & 15u), pv);
                        } else {
                            iw[r] = v + bv;
                        }
                    }
                }
                const bool ok = await_records();
                const uww_chunk_record rec = load_record(&a.records[c]);
                if (ok && !(rec.flags & UWW_CHUNK_OVERFLOW)) {
                    uint32_t* dst = a.inds + rec.ind_offset + bi;
#pragma unroll
                    for (int r = 0; r < (int)(kIndexBlock / 256); ++r) {
                        const uint32_t k = k0 + (uint32_t)r * 256u + tid;
                        if (k < k1) dst[k] = iw[r];
                    }
                }
            } else if (slab) {
                // a slab without staging room: built again in this CTA's
                // scratch, then passes 1 and 2 in place
                if (!await_records()) goto unit_done;
                const uww_chunk_record rec = load_record(&a.records[c]);
                if (rec.flags & UWW_CHUNK_OVERFLOW) goto unit_done;
                emit_slab_again<O>(p, a, T, dyn_smem, c, sl, rec.vert_offset + bv, rec.ind_offset + bi, bv, pv, cnV);
            } else {
                // a chunk without staging room: built again here, then
                // passes 1 and 2 in place
                if (!await_records()) goto unit_done;
                const uww_chunk_record rec = load_record(&a.records[c]);
                if (rec.flags & UWW_CHUNK_OVERFLOW) goto unit_done;
                emit_chunk_again<O>(p, a, T, dyn_smem, c, rec);
            }
        }
    unit_done:
        __syncthreads();  // next_ticket written; the workspace is free
        t = next_ticket;
    }
    // the last CTA: the tile sums and counters left zero for the next launch
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        last = atomicAdd(&a.split_ctr[kCtrDone], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (uint32_t k = tid; k < ntiles; k += nthr) a.tile_sum[k] = 0ull;
    if (tid < kCtrWords) a.split_ctr[tid] = 0u;
    // every error flag of the build: the front kernel's, and a wait of this
    // one that ran out
    if (tid == 0) a.totals[3] = atomicExch(&a.acc[1], 0ull);
}

// Pass 2 of the batched build over every vertex of the batch: vertex counts
// are very uneven across chunks, so the per-vertex colour and analytic-normal
// work is spread over the whole GPU instead of staying with the CTA that
// built the chunk.  The vertex count is read from totals[0].
// totals and verts are written by the build kernel this one may overlap (a
// programmatic dependent): neither is read through the read-only path, and
// nothing is read before griddepcontrol.wait.
template <class O>
__global__ void __launch_bounds__(256) vertex_kernel(const DevParams p, uww_vert_color* verts, float* normals,
                                                     const unsigned long long* totals, uint32_t vert_capacity)
{
    __shared__ __align__(16) uint8_t P[256];
    __shared__ float4 gp[256];
    for (int i = threadIdx.x; i < 64; i += blockDim.x)
        reinterpret_cast<uint32_t*>(P)[i] = reinterpret_cast<const uint32_t*>(p.perm)[i];
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        float gx, gy, gz;
        grad_vec(P[i], gx, gy, gz);
        gp[i] = make_float4(gx, gy, gz, 0.f);
    }
    __syncthreads();
    // launched as a programmatic dependent of the build: wait for all of it
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t nv = (uint32_t)min(__ldcg(totals), (unsigned long long)vert_capacity);
    const bool want_color = (p.outputs & UWW_OUT_COLOR) != 0;
    const bool want_normals = (p.outputs & UWW_OUT_NORMALS) != 0 && normals != nullptr;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
        finish_vertex<O>(p, P, gp, verts, normals, v, want_color, want_normals);
}

// Copy of a build's outputs into host memory the device can address (page-
// locked, mapped): one segment per blockIdx.y, its length fixed or read from
// the build's totals on the device, so the host needs no synchronisation
// between the build and the copies.
__global__ void copy_out_kernel(const CopyOut c, const unsigned long long* __restrict__ totals)
{
    const CopySeg& g = c.seg[blockIdx.y];
    unsigned long long bytes = g.fixed_bytes;
    if (g.count_idx >= 0) bytes = min(totals[g.count_idx], g.cap_elems) * g.elem_bytes;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    const uintptr_t al = (uintptr_t)g.src | (uintptr_t)g.dst;
    if ((al & 15) == 0) {
        // 16-byte words, then the remaining bytes
        const uint4* s4 = reinterpret_cast<const uint4*>(g.src);
        uint4* d4 = reinterpret_cast<uint4*>(g.dst);
        const size_t n16 = bytes / 16;
        for (size_t i = tid; i < n16; i += stride) d4[i] = __ldcs(s4 + i);
        for (size_t i = n16 * 16 + tid; i < bytes; i += stride) g.dst[i] = g.src[i];
    } else if (((al | (uintptr_t)bytes) & 3) == 0) {
        const uint32_t* s1 = reinterpret_cast<const uint32_t*>(g.src);
        uint32_t* d1 = reinterpret_cast<uint32_t*>(g.dst);
        for (size_t i = tid; i < bytes / 4; i += stride) d1[i] = s1[i];
    } else {
        for (size_t i = tid; i < bytes; i += stride) g.dst[i] = g.src[i];
    }
}

template <class O>
__global__ void density_kernel(const DevParams p, const float* __restrict__ xyz, uint32_t n, float* __restrict__ out)
{
    __shared__ __align__(16) uint8_t P[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) P[i] = p.perm[i];
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = density<O, false>(p, P, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], nullptr);
}

using BuildFn = void (*)(const DevParams, const BuildArgs);
using VertexFn = void (*)(const DevParams, uww_vert_color*, float*, const unsigned long long*, uint32_t);

// [exact][queue][large]
BuildFn kernel_for(bool exact, bool queue, bool large)
{
    static const BuildFn table[2][2][2] = {
        {{build_kernel<FastOps, false, 224, 4>, build_kernel<FastOps, false, 544, 1>},
         {build_kernel<FastOps, true, 224, 4>, build_kernel<FastOps, true, 544, 1>}},
        {{build_kernel<ExactOps, false, 224, 4>, build_kernel<ExactOps, false, 544, 1>},
         {build_kernel<ExactOps, true, 224, 4>, build_kernel<ExactOps, true, 544, 1>}}};
    return table[exact][queue][large];
}

size_t set_smem_attr(BuildFn fn, size_t optin)
{
    // The largest dynamic allocation the driver accepts next to this kernel's
    // static shared memory: start from the opt-in limit and step down.
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) return 0;
    size_t want = optin > fa.sharedSizeBytes ? (optin - fa.sharedSizeBytes) & ~size_t(15) : 0;
    for (int i = 0; i < 16 && want >= 1024; ++i, want -= 1024) {
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want) == cudaSuccess)
            return want;
        (void)cudaGetLastError();
    }
    return 0;
}

using FrontFn = void (*)(const DevParams, const BuildArgs);

// The split build's emission kernel.
FrontFn emit_for(bool exact) { return exact ? emit_kernel<ExactOps> : emit_kernel<FastOps>; }

// The split build's front kernel for a CTA of `threads` (<= 256) threads;
// batches with slabs (whose workspaces leave room for two CTAs per SM) take
// the instance with 128 registers a thread.
FrontFn front_for(bool exact, int threads, bool slabs)
{
    if (slabs) return exact ? front_kernel<ExactOps, 256, 2> : front_kernel<FastOps, 256, 2>;
    if (threads <= 192) return exact ? front_kernel<ExactOps, 192, 4> : front_kernel<FastOps, 192, 4>;
    return exact ? front_kernel<ExactOps, 256, 3> : front_kernel<FastOps, 256, 3>;
}

}  // namespace

cudaError_t prepare_build_kernels(size_t optin, size_t* max_dyn_smem)
{
    size_t m = ~size_t(0);
    for (int e = 0; e < 2; ++e) {
        for (int q = 0; q < 2; ++q)
            for (int l = 0; l < 2; ++l) m = std::min(m, set_smem_attr(kernel_for(e, q, l), optin));
        for (int th : {192, 256}) m = std::min(m, set_smem_attr(front_for(e, th, false), optin));
        m = std::min(m, set_smem_attr(front_for(e, 256, true), optin));
        m = std::min(m, set_smem_attr(emit_for(e), optin));
    }
    *max_dyn_smem = m;
    return m >= 16384 ? cudaSuccess : cudaErrorInvalidValue;
}

// Resident CTAs per SM of a kernel at a launch shape, and the device's SM
// count: properties of the device that every batched launch needs, looked up
// once per (device, kernel, threads, dynamic shared memory) and kept, so that
// a build's host side issues its kernels without those queries in between.
cudaError_t occupancy_of(const void* fn, int threads, size_t dyn_smem, int* blocks_per_sm, int* sms = nullptr)
{
    static std::mutex mu;
    static std::map<std::tuple<int, const void*, int, size_t>, int> occ;
    static std::map<int, int> sm_count;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (sms) {
        auto it = sm_count.find(dev);
        if (it == sm_count.end()) {
            int n = 0;
            if ((e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
            it = sm_count.emplace(dev, n).first;
        }
        *sms = it->second;
    }
    const auto key = std::make_tuple(dev, fn, threads, dyn_smem);
    auto it = occ.find(key);
    if (it == occ.end()) {
        int b = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, threads, dyn_smem)) != cudaSuccess) return e;
        it = occ.emplace(key, b).first;
    }
    *blocks_per_sm = it->second;
    return cudaSuccess;
}

cudaError_t build_occupancy(bool queue, bool exact, int threads, size_t dyn_smem, int* blocks_per_sm)
{
    return occupancy_of((const void*)kernel_for(exact, queue, threads > 224), threads, dyn_smem, blocks_per_sm);
}

cudaError_t front_occupancy(bool exact, int threads, size_t dyn_smem, int* blocks_per_sm, bool slabs)
{
    return occupancy_of((const void*)front_for(exact, threads, slabs), threads, dyn_smem, blocks_per_sm);
}

cudaError_t split_emit_shape(const DevParams& p, const BuildArgs& a, int* grid, size_t* dyn_smem)
{
    int sms = 0, ebps = 0;
    // dynamic shared memory: a gathered vertex block (9 words a vertex),
    // the masks and z tables of a whole chunk built again (chunks without
    // staging room; its workspace is in the CTA's scratch slot) or the z
    // tables of a slab built again, the largest
    size_t zt = 0;
    size_t edyn = std::max(rebuild_layout((int)a.smem_cells, (int)p.octaves, p.math_mode != UWW_MATH_EXACT, &zt),
                           (size_t)kVertexBlock * 9 * sizeof(float));
    if (a.pmax > 1) edyn = std::max(edyn, ztable_bytes((int)a.max_cells + 1, (int)p.octaves));
    const cudaError_t e = occupancy_of((const void*)emit_for(p.math_mode == UWW_MATH_EXACT), 256, edyn, &ebps, &sms);
    if (e != cudaSuccess) return e;
    *grid = std::max(1, sms * std::max(1, ebps));
    *dyn_smem = edyn;
    return cudaSuccess;
}

cudaError_t launch_build(const DevParams& p, const BuildArgs& a, bool queue, int grid, int threads, size_t dyn_smem,
                         cudaStream_t s)
{
    const bool exact = p.math_mode == UWW_MATH_EXACT;
    cudaError_t e = cudaSuccess;
    if (queue && a.split) {
        // the split build: [planning ->] front -> emission (-> vertex pass below)
        if (a.split_planned) {
            const uint32_t nblk = std::max(1u, std::min((a.n + kPlanThreads - 1) / kPlanThreads, 1024u));
            split_plan_kernel<<<nblk, kPlanThreads, 0, s>>>(p, a);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = dyn_smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = a.split_planned ? 1 : 0;
        if ((e = cudaLaunchKernelEx(&cfg, front_for(exact, threads, a.pmax > 1), p, a)) != cudaSuccess) return e;
        // the emission (with the records) as the front kernel's programmatic
        // dependent: its CTAs load their tables as front CTAs finish
        cudaLaunchAttribute pdl[1];
        pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        pdl[0].val.programmaticStreamSerializationAllowed = 1;
        int egrid = 0;
        size_t edyn = 0;
        if ((e = split_emit_shape(p, a, &egrid, &edyn)) != cudaSuccess) return e;
        cudaLaunchConfig_t ecfg = {};
        ecfg.gridDim = dim3((unsigned)egrid);
        ecfg.blockDim = dim3(256);
        ecfg.dynamicSmemBytes = edyn;
        ecfg.stream = s;
        ecfg.attrs = pdl;
        ecfg.numAttrs = 1;
        return cudaLaunchKernelEx(&ecfg, emit_for(exact), p, a);
    } else if (queue && a.plan) {
        // the planning kernel, then the build as its programmatic dependent
        const uint32_t nblk = std::max(1u, std::min((a.n + kPlanThreads - 1) / kPlanThreads, 1024u));
        plan_kernel<<<nblk, kPlanThreads, 0, s>>>(p, a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = dyn_smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, kernel_for(exact, queue, threads > 224), p, a);
    } else {
        kernel_for(exact, queue, threads > 224)<<<grid, threads, dyn_smem, s>>>(p, a);
        e = cudaGetLastError();
    }
    // streamed host output finishes its vertices inside the build kernel
    if (e != cudaSuccess || !queue || a.host_verts || !(p.outputs & (UWW_OUT_COLOR | UWW_OUT_NORMALS))) return e;
    // the batched form's pass 2, over the whole batch: one wave of resident
    // CTAs striding over the vertices, launched as a programmatic dependent
    // of the build so that its launch and table setup overlap the build's
    // last CTAs
    int sms = 0;
    const VertexFn vfn = exact ? vertex_kernel<ExactOps> : vertex_kernel<FastOps>;
    int vbps = 0;
    if ((e = occupancy_of((const void*)vfn, 256, 0, &vbps, &sms)) != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)std::max(1, sms * std::max(1, vbps)));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, vfn, p, a.verts, a.normals, (const unsigned long long*)a.totals, a.vert_capacity);
}

size_t table_image_bytes() { return kTableImageBytes; }

cudaError_t launch_table_image(const DevParams& p, void* out, cudaStream_t s)
{
    table_image_kernel<<<1, 256, 0, s>>>(p, static_cast<uint2*>(out));
    return cudaGetLastError();
}

cudaError_t launch_copy_out(const CopyOut& c, const unsigned long long* totals, int blocks_x, cudaStream_t s)
{
    if (c.nseg <= 0) return cudaSuccess;
    copy_out_kernel<<<dim3((unsigned)blocks_x, (unsigned)c.nseg), 256, 0, s>>>(c, totals);
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
