// uww_internal.h -- host/device shared declarations of libuww_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "uww.h"
#include "uww_device.cuh"

namespace uww {

// Per-chunk working set, in shared memory when it fits, else in a global
// scratch slot owned by the CTA.  Offsets are 16-byte aligned.
struct ChunkLayout {
    uint32_t rho;      // (N+1)^3 f32 samples, index (x*S + y)*S + z
    uint32_t cases;    // N^3 u8 case indices, cell order x, y, z
    uint32_t vbase;    // N^3: first chunk-local vertex id created by each cell (u16 when idx16)
    uint32_t active;   // active-cell list (u16 when active16)
    uint32_t ibase;    // per active cell: first index position (u16 when idx16)
    uint32_t total;
    bool active16;
    bool idx16;
};

__host__ __device__ inline uint32_t align16(uint32_t v) { return (v + 15u) & ~15u; }

__host__ __device__ inline ChunkLayout chunk_layout(int N)
{
    ChunkLayout L;
    const uint32_t S = (uint32_t)N + 1, NC = (uint32_t)N * N * N;
    L.active16 = NC <= 65536u;
    // at most 15 indices per cell, and fewer vertices than indices
    L.idx16 = 15u * NC < 65536u;
    const uint32_t ib = L.idx16 ? 2u : 4u;
    uint32_t o = 0;
    L.rho = o;    o = align16(o + S * S * S * 4u);
    L.cases = o;  o = align16(o + NC);
    L.vbase = o;  o = align16(o + NC * ib);
    L.active = o; o = align16(o + NC * (L.active16 ? 2u : 4u));
    L.ibase = o;  o = align16(o + NC * ib);
    L.total = o;
    return L;
}

// Split build, chunks above 16 cells per edge (the 24^3 and 48^3 LODs): each is
// built as slabs of K consecutive x layers of cells -- contiguous in the
// chunk's cell order (x, y, z), so a chunk's output is its slabs' outputs in
// slab order -- one CTA of kSlabThreads threads per slab.  A slab's shared
// workspace: the samples of its K+1 x planes, per sample column its
// below-iso bits, per cell its case and (active cells) its first vertex id
// within the slab, and the list of its active cells (up to kSlabActCap:
// cell | first triangle << 16) that spreads pass 1 over the CTA.  K is
// the largest layer count whose sample columns ((K+1) * S) fit one pass of the
// CTA's threads, whose workspace fits kSlabBudget bytes, and whose vertices fit
// 16-bit ids (slab_vertex_bound).
constexpr int kSlabThreads = 256;
constexpr uint32_t kSlabBudget = 96 * 1024;
constexpr uint32_t kSlabActCap = 2048;
constexpr int kSlabMaxCells = 63;     // a sample column's bits fit one 64-bit mask
constexpr uint32_t kPieceShift = 24;  // queue entry: chunk | slab << kPieceShift

struct SlabLayout {
    uint32_t rho, cases, vbase, masks, alist, total;
    int K;
};

__host__ __device__ inline SlabLayout slab_layout_k(int N, int K)
{
    const uint32_t S = (uint32_t)N + 1, NC = (uint32_t)K * N * N;
    SlabLayout L;
    L.K = K;
    uint32_t o = 0;
    L.rho = o;    o = align16(o + (uint32_t)(K + 1) * S * S * 4u);
    L.cases = o;  o = align16(o + NC);
    L.vbase = o;  o = align16(o + NC * 2u);
    L.masks = o;  o = align16(o + (uint32_t)(K + 1) * S * 8u);
    L.alist = o;  o = align16(o + kSlabActCap * 4u);
    L.total = o;
    return L;
}

// The most vertices a slab of K layers of an N-cell chunk can create, in
// either dedup mode: with one vertex per cube edge, every edge of its cells
// once, K S^2 + 2 (K+1) N S; with one per ordered corner pair (the
// reference's), the cells on either side of an x or a z edge list it with
// opposite corner order, so those edges can carry two vertices and y edges
// one, (5K+1) N S -- the larger.  Both are reached when every edge is crossed.
__host__ __device__ inline long long slab_vertex_bound(int N, int K)
{
    const long long S = N + 1;
    const long long edges = (long long)K * S * S + 2ll * (K + 1) * N * S;
    const long long oriented = (5ll * K + 1) * N * S;
    return edges > oriented ? edges : oriented;
}

__host__ __device__ inline int slab_layers(int N)
{
    const int S = N + 1;
    int K = kSlabThreads / S - 1;
    if (K > N) K = N;
    for (; K > 1; --K)
        if (slab_layout_k(N, K).total <= kSlabBudget && slab_vertex_bound(N, K) < 65536) break;
    return K < 1 ? 1 : K;
}

__host__ __device__ inline SlabLayout slab_layout(int N) { return slab_layout_k(N, slab_layers(N)); }
__host__ __device__ inline int slab_count(int N)
{
    const int K = slab_layers(N);
    return (N + K - 1) / K;
}

// Bytes of the fast build's per-chunk z tables for S samples per edge:
// (dz, fade) and (first z, cell) per octave and z, run counts, z bias, run
// start masks.
__host__ __device__ inline size_t ztable_bytes(int S, int octaves)
{
    return (size_t)octaves * S * (sizeof(float2) + sizeof(int2)) + (size_t)octaves * sizeof(int) +
           (size_t)S * sizeof(float) + (size_t)octaves * sizeof(unsigned) + 16;
}

// The split build's emission kernel builds a whole chunk again (one the
// staging buffers had no room for, of up to `cells` cells per edge) with its
// workspace in the CTA's global scratch slot; its dynamic shared memory holds
// (fast build) the chunk's column masks and, at *zt_off, its z tables.
// Returns those bytes.
__host__ __device__ inline size_t rebuild_layout(int cells, int octaves, bool fast, size_t* zt_off)
{
    const size_t S = (size_t)cells + 1;
    *zt_off = fast ? ((S * S * 8 + 15) & ~size_t(15)) : 0;
    return fast ? *zt_off + ztable_bytes((int)S, octaves) : 0;
}

// Plan buffer of a planned batched build of n chunks: u32 [0] the planning
// kernel's finish counter (zero between launches, at a fixed place whatever
// n), [1] the number of listed chunks, [2 .. n+1] the listed chunks in
// order, then one decision byte per chunk.
constexpr uint32_t kPlanDone = 0, kPlanCount = 1, kPlanList = 2;
__host__ __device__ inline size_t plan_kinds_offset(uint32_t n) { return ((size_t)n + kPlanList) * sizeof(uint32_t); }
__host__ __device__ inline size_t plan_buffer_bytes(uint32_t n) { return plan_kinds_offset(n) + n; }

// Split build (uww_build.cu): chunks per tile of the tile sums (the emission
// kernel scans a tile with one warp, a lane per chunk), vertices and indices per
// emission unit, cost ranks of the planning kernel's work queues, and the
// words of the counter block: [kCtrQueued + r] chunks queued at rank r,
// [kCtrTaken + r] taken from queue r, the units in list A (vertex blocks,
// whole chunks) and list B (index blocks), the units taken, the emission
// CTAs finished, (u64 at word kCtrStage) the staging buffers' fill,
// vertices | indices << 32, and the record tiles written.  All zero between
// launches.
constexpr uint32_t kTileChunks = 32;
constexpr uint32_t kVertexBlock = 256, kIndexBlock = 2048;
constexpr int kPlanRanks = 8;
constexpr uint32_t kCtrQueued = 0, kCtrTaken = 8, kCtrUnitsA = 16, kCtrUnitsB = 17, kCtrUnitsTaken = 18,
                   kCtrDone = 19, kCtrStage = 20, kCtrRecDone = 22, kCtrWords = 32;

// Lookback word: [63:62] status, [61:30] indices, [29:0] vertices.
constexpr unsigned long long kLbAggregate = 1ull << 62;
constexpr unsigned long long kLbInclusive = 2ull << 62;
constexpr unsigned long long kLbVertMax = (1ull << 30) - 1;
constexpr unsigned long long kLbIndMax = (1ull << 32) - 1;

// totals[3] error bits
constexpr unsigned long long kErrTimeout = UWW_ERRFLAG_TIMEOUT;
constexpr unsigned long long kErrBadChunk = UWW_ERRFLAG_BAD;
constexpr unsigned long long kErrRange = UWW_ERRFLAG_RANGE;

struct BuildArgs {
    const uww_chunk_desc* chunks;
    uint32_t n;
    uint32_t max_cells;
    uww_vert_color* verts;
    float* normals;
    uint32_t* inds;
    uint8_t* cases;
    float* samples_out;              // optional copy of each chunk's density samples
    const float* samples_in;         // when set, samples are read instead of computed
    unsigned long long case_capacity;     // bytes at cases
    unsigned long long sample_capacity;   // floats at samples_out
    unsigned long long samples_in_count;  // floats at samples_in
    uww_chunk_record* records;
    unsigned long long* totals;      // never NULL inside the kernel
    uint32_t vert_capacity;
    uint32_t ind_capacity;
    unsigned long long* lookback;    // n words, zero at launch; the last CTA re-zeroes them (queue mode)
    unsigned int* work_counter;      // zero at launch; reset by the last CTA (queue mode)
    unsigned long long* acc;         // [0] overflow count, [1] error flags, [2] CTAs finished (queue mode)
    uint8_t* scratch;                // per-CTA slots: chunks above smem_cells (pipelined), rebuilds (split emission)
    size_t scratch_slot_bytes;
    uint32_t slots_per_cta;          // workspaces per CTA (2 in the pipelined batched form)
    size_t smem_buf_bytes;           // bytes of one shared-memory workspace
    size_t ztable_offset;            // fast build: per-chunk z tables, after the workspaces
    uint32_t smem_cells;             // chunks with cells <= smem_cells work in shared memory
    long long spin_limit_cycles;     // bound on every device-side wait
    uint32_t withhold_first;         // UWW_TEST_WITHHOLD_FIRST: ticket 0 never publishes its prefix
    uint32_t withhold_records;       // UWW_TEST_WITHHOLD_RECORDS: tile 0's records are never announced
    uint32_t no_depth_shortcut;      // UWW_TUNE_NO_DEPTH_SHORTCUT: every chunk evaluates its noise
    uint32_t* edge_ids;              // optional, per output vertex: (first corner sample << 3) | direction
    const uint32_t* n_dev;           // optional device chunk count; the launch builds min(*n_dev, n)
    uint32_t* plan;                  // planned batch: finish counter, count, list (plan_kernel; kPlan*)
    // Split build (every chunk or slab in shared memory, no streamed host
    // output).  Per chunk c: its counts word tinfo[c] (packed counts,
    // early-blank flag in bit 62) and, when meshed, where its staged pass 1
    // sits (stage_at[c * pmax]: vertices | indices << 32; all ones when the
    // staging buffers had no room -- the emission kernel then builds it
    // again); per tile of kTileChunks chunks the sum of its counts
    // (verts | inds << 32).
    uint32_t split;                  // the split build (planning, front and emission kernels)
    unsigned long long* tinfo;
    unsigned long long* tile_sum;    // zero at launch; re-zeroed by the emission kernel's last CTA
    unsigned long long* stage_at;
    float4* stage_pos;               // staging: per vertex position and corner b
    uint32_t* stage_inds;            // staging: chunk-local indices
    uint32_t stage_vcap, stage_icap;
    unsigned long long* stage_ctr;   // the staging fill (counter block word kCtrStage)
    unsigned long long* units;       // emission units (unit_entry): list A from the front, list B from the back
    uint32_t unit_cap;
    uint32_t* split_queue;           // planned: kPlanRanks work queues of n * pmax entries
    uint32_t* split_ctr;             // kCtrWords counters, zero at launch (kCtr*)
    uint32_t split_planned;          // the planning kernel runs first and fills the queues
    uint32_t split_decide;           // ... and settles the chunks the depth bias decides (else queues every chunk)
    uint32_t* stage_eids;            // staging: per vertex its edge id (when edge_ids is set)
    uint32_t mask_offset;            // nonzero: per-column below-iso masks at dyn smem + mask_offset
    const uint2* tables;             // optional: the marching-cubes table image (table_image_kernel)
    // Slabs (chunks above piece_cells cells per edge, split build): a chunk
    // has pmax piece places p = c * pmax + s.  Per place its counts (pinfo:
    // verts | inds << 32), its staging place (stage_at[p]) and the seam it
    // leaves its successor (seam + p * seam_stride words: per cell (y, z) of
    // its last layer, the cell's first vertex id within the slab | case <<
    // 16); a slab built again by the emission kernel works in scratch +
    // blockIdx.x * scratch_slot_bytes.  pmax == 1: no slabs; every place is a
    // chunk.
    uint32_t pmax;
    uint32_t piece_cells;
    unsigned long long* pinfo;
    uint32_t* seam;
    uint32_t seam_stride;
    // Optional streamed host output (batched form): device addresses of
    // page-locked host memory.  Pass 2 then runs inside the build kernel, and
    // each chunk's record, indices, vertices and normals go there as soon as
    // the chunk is finished (`verts`, `normals` and `inds` still receive the
    // output), so the transfer to the host overlaps the build.
    uint32_t* host_inds;
    uww_chunk_record* host_records;
    uww_vert_color* host_verts;
    float* host_normals;
    unsigned long long* host_totals;  // optional copy of the four totals, by the last CTA (queue mode)
};

// Device -> mapped-host copy of a build's outputs (uww_build.cu).
struct CopySeg {
    const uint8_t* src;
    uint8_t* dst;                    // device address of page-locked host memory
    unsigned long long fixed_bytes;  // when count_idx < 0
    int count_idx;                   // else bytes = min(totals[count_idx], cap_elems) * elem_bytes
    uint32_t elem_bytes;
    unsigned long long cap_elems;
};
struct CopyOut {
    CopySeg seg[8];
    int nseg;
};
cudaError_t launch_copy_out(const CopyOut& c, const unsigned long long* totals, int blocks_x, cudaStream_t s);
// The build kernels' marching-cubes tables in shared-memory layout, as one
// image in device memory (table_image_bytes() bytes at out), the same for
// every parameter set.
size_t table_image_bytes();
cudaError_t launch_table_image(const DevParams& p, void* out, cudaStream_t s);

// Host helpers shared by the entry points (uww_api.cu).
int check_params(const uww_params* p);
void dev_params_from(const uww_params* p, DevParams* d);
int status_from_cuda(cudaError_t e, const char* where);  // records the CUDA error text
long long spin_limit_cycles();
// compute threads per CTA for a batch whose largest chunk has max_cells per edge
int default_compute_threads(uint32_t max_cells);

// Launch helpers (uww_build.cu).
cudaError_t launch_build(const DevParams& p, const BuildArgs& a, bool queue, int grid, int threads,
                         size_t dyn_smem, cudaStream_t s);
cudaError_t build_occupancy(bool queue, bool exact, int threads, size_t dyn_smem, int* blocks_per_sm);
// the split build's front kernel: resident CTAs per SM for this shape
cudaError_t front_occupancy(bool exact, int threads, size_t dyn_smem, int* blocks_per_sm, bool slabs = false);
cudaError_t prepare_build_kernels(size_t optin, size_t* max_dyn_smem);
// the split build's emission kernel: its grid and dynamic shared memory
cudaError_t split_emit_shape(const DevParams& p, const BuildArgs& a, int* grid, size_t* dyn_smem);
cudaError_t launch_density(const DevParams& p, const float* xyz, uint32_t n, float* out, cudaStream_t s);

// Batched build on the context (uww_api.cu); edge_ids and n_dev as in BuildArgs.
int launch_batched(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                   const uww_mesh_out* out, uint32_t* edge_ids, const uint32_t* n_dev);
int check_mesh_out(const uww_mesh_out* out);
// allocate what a batched build of n chunks needs, without launching (so that
// a later launch can be captured into a CUDA graph)
int prepare_batched(uww_ctx* ctx, uint32_t n, uint32_t max_cells, const uww_mesh_out* out);
// the launch shape a batched build of n chunks would use
// and the resident CTAs per SM of its (front) kernel
int plan_batched(uww_ctx* ctx, uint32_t n, uint32_t max_cells, int* threads, int* grid, size_t* dyn_smem,
                 int* occupancy, uint32_t* split = nullptr, uint32_t* pmax = nullptr);
// (re)allocate *ptr to at least `bytes` of device memory (contents not kept)
int ensure_device_bytes(void** ptr, size_t* cap, size_t bytes);
// The build writes vertex positions and the totals with 8-byte stores and
// everything else (descriptors read) with 4-byte words: device buffers that
// are not aligned to match are refused with UWW_ERR_INVALID_ARG before any
// launch, instead of faulting in the kernel.
inline bool aligned_to(const void* p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) == 0; }
inline bool device_out_aligned(const uww_mesh_out* o)
{
    return aligned_to(o->verts, 8) && aligned_to(o->normals, 4) && aligned_to(o->inds, 4) &&
           aligned_to(o->records, 4) && aligned_to(o->totals, 8) && aligned_to(o->samples, 4);
}

template <class T>
int ensure_device_of(T** ptr, size_t* cap, size_t bytes)
{
    return ensure_device_bytes(reinterpret_cast<void**>(ptr), cap, bytes);
}

}  // namespace uww

// The context behind the opaque uww_ctx handle.
struct uww_ctx {
    uww_params params;
    uww::DevParams dev;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    size_t smem_dyn_max = 0;

    // tuning (0 = automatic)
    int threads = 0;
    int blocks_per_sm = 0;
    int smem_cells = 0;
    long long spin_limit = 0;     // bound on device-side waits in cycles; 0 = kSpinLimitCycles
    uint32_t test_flags = 0;      // UWW_TEST_* failure injection
    uint32_t options = 0;         // UWW_TUNE_*

    // device work state
    unsigned long long* d_lookback = nullptr;
    size_t lookback_cap = 0;
    uint32_t* d_plan = nullptr;   // planned batch: chunk count + list
    size_t plan_cap = 0;
    void* d_tables = nullptr;     // the marching-cubes table image (launch_table_image)
    uint8_t* d_split = nullptr;   // split build: counters, tile sums, counts, staging places, queues
    uint8_t* d_stage = nullptr;   // split build: staging buffers and emission units
    uint8_t* d_slab = nullptr;    // split build with slabs: per place its counts, then its seam
    size_t slab_cap = 0;
    size_t stage_cap = 0;
    size_t split_cap = 0;
    uint32_t split_n = 0;         // the chunk count its layout is made for
    unsigned long long* d_state = nullptr;
    unsigned int* d_counter = nullptr;
    unsigned long long* d_acc = nullptr;
    unsigned long long* d_totals = nullptr;
    uint8_t* d_scratch = nullptr;
    size_t scratch_cap = 0;
    uint64_t work_gen = 0;  // moves on whenever d_scratch or d_lookback is reallocated

    // buffers of the host-buffer path
    uww_chunk_desc* d_chunks = nullptr;
    size_t chunks_cap = 0;
    void* d_verts = nullptr;     size_t verts_cap = 0;
    void* d_normals = nullptr;   size_t normals_cap = 0;
    void* d_inds = nullptr;      size_t inds_cap = 0;
    void* d_cases = nullptr;     size_t cases_cap = 0;
    void* d_samples = nullptr;   size_t samples_cap = 0;
    void* d_records = nullptr;   size_t records_cap = 0;
    unsigned long long* h_totals = nullptr;

    // adjoint: per-chunk dL/dtheta partials and the arrival counter of the
    // backward's final reduction (zero between launches)
    float* d_adj_part = nullptr;     size_t adj_part_cap = 0;
    unsigned int* d_adj_counter = nullptr;
    // uww_sample_chunks: UWW_ERRFLAG_* of the last call
    unsigned int* d_sample_err = nullptr;
};