// uww_api.cu -- the C ABI (include/uww.h): contexts, parameter handling,
// the seeded permutation, launch configuration and the host-buffer path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "uww_internal.h"

using namespace uww;

// struct uww_ctx is defined in uww_internal.h (shared with the adjoint and tuner).


namespace {

constexpr long long kSpinLimitCycles = 4000000000ll;  // ~2 s at 2 GHz

thread_local char g_last_error[256] = "";

void note_error(const char* where, cudaError_t e)
{
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%d)", where, cudaGetErrorString(e), (int)e);
}

int cuda_status(cudaError_t e, const char* where = "CUDA call")
{
    if (e == cudaSuccess) return UWW_OK;
    note_error(where, e);
    return e == cudaErrorMemoryAllocation ? UWW_ERR_OOM : UWW_ERR_CUDA;
}

// --- noise::Perlin::new(seed) permutation --------------------------------------
// The crate seeds an XorShift128 generator with the bytes
// [1,0,0,0, seed x3] (x = 1, y = z = w = seed) and shuffles 0..255 with
// rand's Fisher-Yates (i from 255 down to 1, j uniform in [0, i]); the
// bounded draw multiplies a 32-bit output by the range and rejects low
// words above (range << clz(range)) - 1.
struct XorShift128 {
    uint32_t x, y, z, w;
    uint32_t next()
    {
        const uint32_t t = x ^ (x << 11);
        x = y; y = z; z = w;
        w = w ^ (w >> 19) ^ (t ^ (t >> 8));
        return w;
    }
    uint32_t below(uint32_t range)
    {
        const uint32_t zone = (range << __builtin_clz(range)) - 1u;
        for (;;) {
            const uint64_t m = (uint64_t)next() * range;
            if ((uint32_t)m <= zone) return (uint32_t)(m >> 32);
        }
    }
};

void make_perm(uint32_t seed, uint8_t out[256])
{
    XorShift128 r{1u, seed, seed, seed};
    for (int i = 0; i < 256; ++i) out[i] = (uint8_t)i;
    for (uint32_t i = 255; i >= 1; --i) std::swap(out[i], out[r.below(i + 1)]);
}

bool finite(float v) { return std::isfinite(v); }

int validate_params(const uww_params* p)
{
    if (!p) return UWW_ERR_INVALID_ARG;
    if (p->octaves < 1 || p->octaves > UWW_MAX_OCTAVES) return UWW_ERR_INVALID_ARG;
    if (p->chunk_size < 1 || p->chunk_size > (1 << 20)) return UWW_ERR_INVALID_ARG;
    if (!finite(p->base_freq) || !finite(p->lacunarity) || !finite(p->persistence) || !finite(p->amplitude))
        return UWW_ERR_INVALID_ARG;
    if (!finite(p->iso_level) || !finite(p->offset[0]) || !finite(p->offset[1]) || !finite(p->offset[2]))
        return UWW_ERR_INVALID_ARG;
    if (!finite(p->bias_a) || !finite(p->bias_b) || !finite(p->bias_c)) return UWW_ERR_INVALID_ARG;
    if (!finite(p->color_min_z) || !finite(p->color_max_z)) return UWW_ERR_INVALID_ARG;
    if (p->outputs & ~(UWW_OUT_COLOR | UWW_OUT_NORMALS | UWW_OUT_CASES | UWW_OUT_SAMPLES)) return UWW_ERR_INVALID_ARG;
    if (p->bias_mode < UWW_BIAS_NONE || p->bias_mode > UWW_BIAS_LINEAR) return UWW_ERR_INVALID_ARG;
    if (p->bias_mode == UWW_BIAS_TERRACED && (p->bias_b == 0.f || p->bias_c == 0.f)) return UWW_ERR_INVALID_ARG;
    if (p->math_mode != UWW_MATH_EXACT && p->math_mode != UWW_MATH_FAST) return UWW_ERR_INVALID_ARG;
    if (p->dedup_mode != UWW_DEDUP_ORIENTED && p->dedup_mode != UWW_DEDUP_EDGE) return UWW_ERR_INVALID_ARG;
    if (p->color_max_z == p->color_min_z) return UWW_ERR_INVALID_ARG;
    if (p->explicit_amps)
        for (uint32_t k = 0; k < p->octaves; ++k)
            if (!finite(p->amps[k])) return UWW_ERR_INVALID_ARG;
    return UWW_OK;
}

void make_dev_params(const uww_params* p, DevParams* d)
{
    std::memset(d, 0, sizeof(*d));
    make_perm(p->seed, d->perm);
    // perlin_util.rs:8-20: frequency and amplitude advance by repeated f32 multiplies
    float m = 1.f, a = p->amplitude;
    for (uint32_t k = 0; k < p->octaves; ++k) {
        d->mult[k] = m;
        d->amp[k] = p->explicit_amps ? p->amps[k] : a;
        m = m * p->lacunarity;
        a = a * p->persistence;
    }
    d->octaves = (int32_t)p->octaves;
    d->chunk_size = p->chunk_size;
    d->base_freq = p->base_freq;
    d->iso_level = p->iso_level;
    for (int i = 0; i < 3; ++i) d->offset[i] = p->offset[i];
    d->normalize = p->normalize;
    d->bias_mode = p->bias_mode;
    d->bias_a = p->bias_a;
    d->bias_b = p->bias_b;
    d->bias_c = p->bias_c;
    d->color_min_z = p->color_min_z;
    d->color_max_z = p->color_max_z;
    d->outputs = p->outputs;
    d->dedup_mode = p->dedup_mode;
    d->math_mode = p->math_mode;
}

template <class T>
int ensure_device(T** ptr, size_t* cap, size_t bytes)
{
    if (*cap >= bytes && *ptr) return UWW_OK;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    *cap = 0;
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc((void**)ptr, want);
    if (e != cudaSuccess) { *ptr = nullptr; return cuda_status(e); }
    *cap = want;
    return UWW_OK;
}

struct LaunchCfg {
    int threads;
    uint32_t smem_cells;
    uint32_t slots;        // workspaces per CTA
    size_t smem_buf;       // bytes of one shared-memory workspace
    size_t ztable_offset;  // fast build z tables, after the workspaces
    size_t dyn_smem;
    int grid;
    int occupancy;         // resident CTAs per SM of the build's (front) kernel
    uint32_t mask_offset;  // split front kernel: column masks in dynamic shared memory (0: none)
    size_t scratch_slot;
    bool split;            // the split build: front kernel, then emission over every triangle
    uint32_t pmax;         // split build: places per chunk (> 1: chunks above 16 cells are built as slabs)
    size_t slab_slot;      // bytes of the largest slab workspace (the emission's per-CTA scratch)
};

// Whether a batched build is planned (a first kernel decides chunks by their
// depth bias and queues the rest): nothing reads or writes its samples or
// cases, and the depth shortcut is on.
bool plans(const uww_ctx* ctx, const uww_mesh_out* out, const float* samples_in)
{
    const bool samples_out = (ctx->params.outputs & UWW_OUT_SAMPLES) && (!out || out->samples);
    const bool cases = (ctx->params.outputs & UWW_OUT_CASES) && (!out || out->cases);
    return !samples_in && !samples_out && !cases && !(ctx->options & UWW_TUNE_NO_DEPTH_SHORTCUT);
}

// split_ok: nothing of the launch needs the pipelined kernel (streamed host
// output and per-vertex edge ids do)
int plan_launch(uww_ctx* ctx, uint32_t n, uint32_t max_cells, bool queue, LaunchCfg* cfg, bool split_ok, bool planned,
                bool samples_in = false)
{
    const size_t cap = ctx->smem_dyn_max;
    const int compute = ctx->threads > 0 ? ctx->threads : default_compute_threads(max_cells);
    const size_t zt_max = ctx->dev.math_mode == UWW_MATH_FAST ? ztable_bytes((int)max_cells + 1, ctx->dev.octaves) : 0;
    cfg->pmax = 1;
    cfg->slab_slot = 0;
    // A batch with chunks above 16 cells per edge (the 24^3 and 48^3 LODs)
    // whose samples are computed, not read: the split build, with those
    // chunks as slabs of a few x layers (one CTA of kSlabThreads threads
    // each) and the rest whole, in one shared workspace sized for the larger
    // of a 16^3 chunk and a slab.
    (void)planned;
    if (queue && split_ok && !samples_in && max_cells > 16 && max_cells <= (uint32_t)kSlabMaxCells &&
        n < (1u << kPieceShift) && !(ctx->options & UWW_TUNE_PIPELINED) &&
        !(ctx->test_flags & UWW_TEST_WITHHOLD_FIRST) && ctx->smem_cells <= 0 &&
        (ctx->threads <= 0 || ctx->threads == kSlabThreads)) {
        uint32_t slab_bytes = 0;
        int pmax = 1;
        for (int N = 17; N <= (int)max_cells; ++N) {
            slab_bytes = std::max(slab_bytes, slab_layout(N).total);
            pmax = std::max(pmax, slab_count(N));
        }
        const size_t ws = std::max<size_t>(chunk_layout(16).total, slab_bytes);
        size_t dyn = ws + zt_max;
        uint32_t mo = 0;
        if (ctx->dev.math_mode == UWW_MATH_FAST) {
            mo = (uint32_t)((dyn + 15) & ~size_t(15));
            dyn = mo + 13 * 13 * sizeof(unsigned long long);
        }
        if (dyn <= cap) {
            cfg->split = true;
            cfg->pmax = (uint32_t)pmax;
            cfg->slab_slot = align16(slab_bytes);
            cfg->smem_cells = 16;
            cfg->slots = 1;
            cfg->smem_buf = ws;
            cfg->ztable_offset = ws;
            cfg->dyn_smem = dyn;
            cfg->mask_offset = mo;
            cfg->threads = kSlabThreads;
            cfg->scratch_slot = 0;
            const bool exact = ctx->dev.math_mode == UWW_MATH_EXACT;
            cudaError_t e = front_occupancy(exact, cfg->threads, cfg->dyn_smem, &cfg->occupancy, true);
            if (e != cudaSuccess) return cuda_status(e);
            const int bps = ctx->blocks_per_sm > 0 ? ctx->blocks_per_sm : cfg->occupancy;
            if (bps < 1) return UWW_ERR_INVALID_ARG;
            cfg->grid = (int)std::min<long long>((long long)bps * ctx->num_sms, (long long)n * pmax);
            return UWW_OK;
        }
    }
    // A batch whose every chunk fits one shared-memory workspace is built in
    // two kernels (the front half of every chunk, then the emission of every
    // triangle); the look-back test flag and the PIPELINED option keep the
    // single pipelined kernel.
    cfg->split = queue && split_ok && compute <= 256 && !(ctx->options & UWW_TUNE_PIPELINED) &&
                 !(ctx->test_flags & UWW_TEST_WITHHOLD_FIRST) &&
                 (ctx->smem_cells <= 0 || (uint32_t)ctx->smem_cells >= max_cells) &&
                 chunk_layout((int)max_cells).total + zt_max <= cap;
    // The pipelined batched form keeps two chunks per CTA in flight, so it
    // holds two workspaces.
    const uint32_t slots = (queue && !cfg->split) ? 2u : 1u;
    // by default chunks up to 16 cells work in shared memory; a batch with
    // larger ones keeps 12 there (small workspaces, more CTAs per SM) and the
    // rest in global scratch -- except in the split build, where every chunk
    // does
    uint32_t smem_cells = cfg->split               ? max_cells
                          : ctx->smem_cells > 0    ? (uint32_t)ctx->smem_cells
                          : max_cells > 16         ? 12u
                                                   : max_cells;
    smem_cells = std::min(smem_cells, max_cells);
    // the fast build also keeps per-chunk z tables (sized for the largest chunk)
    const size_t zt = zt_max;
    while (smem_cells > 0 && (size_t)slots * chunk_layout((int)smem_cells).total + zt > cap) --smem_cells;
    cfg->smem_cells = smem_cells;
    cfg->slots = slots;
    cfg->smem_buf = smem_cells > 0 ? chunk_layout((int)smem_cells).total : 0;
    cfg->ztable_offset = (size_t)slots * cfg->smem_buf;
    cfg->dyn_smem = cfg->ztable_offset + zt;
    // the split front kernel's 13^3-sample chunks (register-column noise)
    // also keep each column's below-iso mask, for the classification
    cfg->mask_offset = 0;
    if (cfg->split && ctx->dev.math_mode == UWW_MATH_FAST && max_cells == 12) {
        const size_t mo = (cfg->dyn_smem + 15) & ~size_t(15);
        if (mo + 13 * 13 * sizeof(unsigned long long) <= cap) {
            cfg->mask_offset = (uint32_t)mo;
            cfg->dyn_smem = mo + 13 * 13 * sizeof(unsigned long long);
        }
    }
    // compute threads: by default 192 for chunks of up to 12 cells (one per
    // sample column of a 13^3 grid), 256 up to 16 cells (two CTAs per SM) and
    // 512 above (one CTA per SM: a 25^2-column chunk in global scratch is
    // latency-bound, 1.7x faster than with 256); the batched form adds one
    // control warp
    cfg->threads = compute + ((queue && !cfg->split) ? 32 : 0);
    cfg->scratch_slot = max_cells > smem_cells ? chunk_layout((int)max_cells).total : 0;
    cfg->occupancy = 0;
    if (!queue) {
        cfg->grid = 1;
        return UWW_OK;
    }
    const bool exact = ctx->dev.math_mode == UWW_MATH_EXACT;
    cudaError_t e = cfg->split ? front_occupancy(exact, cfg->threads, cfg->dyn_smem, &cfg->occupancy)
                               : build_occupancy(true, exact, cfg->threads, cfg->dyn_smem, &cfg->occupancy);
    if (e != cudaSuccess) return cuda_status(e);
    int bps = ctx->blocks_per_sm > 0 ? ctx->blocks_per_sm : cfg->occupancy;
    if (bps < 1) return UWW_ERR_INVALID_ARG;
    const long long g = (long long)bps * ctx->num_sms;
    cfg->grid = (int)std::min<long long>(g, n);
    return UWW_OK;
}

// Device addresses of page-locked host buffers for the streamed host output
// of a batched build (BuildArgs::host_*).
struct HostOut {
    uww_vert_color* verts;
    float* normals;
    uint32_t* inds;
    uww_chunk_record* records;
    unsigned long long* totals;
};

int launch(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells, const uww_mesh_out* out,
           bool queue, const float* samples_in = nullptr, unsigned long long samples_in_count = 0,
           uint32_t* edge_ids = nullptr, const uint32_t* n_dev = nullptr, bool prepare_only = false,
           const HostOut* host = nullptr)
{
    LaunchCfg cfg;
    int st = plan_launch(ctx, n, max_cells, queue, &cfg, host == nullptr, plans(ctx, out, samples_in),
                         samples_in != nullptr);
    if (st) return st;
    // the work buffers a captured frame graph refers to: a reallocation
    // moves the context's generation on, and such a frame recaptures itself
    auto grow = [ctx](auto** ptr, size_t* cap, size_t bytes) {
        const void* old = *ptr;
        const int r = ensure_device(ptr, cap, bytes);
        if (*ptr != old) ++ctx->work_gen;
        return r;
    };
    if (cfg.scratch_slot) {
        st = grow(&ctx->d_scratch, &ctx->scratch_cap, cfg.scratch_slot * cfg.slots * (size_t)cfg.grid);
        if (st) return st;
    }
    if (prepare_only && !queue) return UWW_OK;
    BuildArgs a;
    std::memset(&a, 0, sizeof(a));
    a.chunks = d_chunks;
    a.n = n;
    a.max_cells = max_cells;
    a.verts = out->verts;
    a.normals = out->normals;
    a.inds = out->inds;
    a.cases = out->cases;
    a.samples_out = (ctx->params.outputs & UWW_OUT_SAMPLES) ? out->samples : nullptr;
    a.samples_in = samples_in;
    a.samples_in_count = samples_in_count;
    a.case_capacity = out->case_capacity;
    a.sample_capacity = out->sample_capacity;
    a.records = out->records;
    a.totals = out->totals ? reinterpret_cast<unsigned long long*>(out->totals) : ctx->d_totals;
    a.vert_capacity = out->vert_capacity;
    a.ind_capacity = out->ind_capacity;
    a.scratch = ctx->d_scratch;
    a.scratch_slot_bytes = cfg.scratch_slot;
    a.slots_per_cta = cfg.slots;
    a.smem_buf_bytes = cfg.smem_buf;
    a.ztable_offset = cfg.ztable_offset;
    a.mask_offset = cfg.mask_offset;
    a.tables = static_cast<const uint2*>(ctx->d_tables);
    a.smem_cells = cfg.smem_cells;
    a.spin_limit_cycles = ctx->spin_limit > 0 ? ctx->spin_limit : kSpinLimitCycles;
    a.withhold_first = (ctx->test_flags & UWW_TEST_WITHHOLD_FIRST) ? 1u : 0u;
    a.withhold_records = (ctx->test_flags & UWW_TEST_WITHHOLD_RECORDS) ? 1u : 0u;
    a.no_depth_shortcut = (ctx->options & UWW_TUNE_NO_DEPTH_SHORTCUT) ? 1u : 0u;
    a.edge_ids = edge_ids;
    a.n_dev = n_dev;
    if (host && queue) {
        a.host_verts = host->verts;
        a.host_normals = host->normals;
        a.host_inds = host->inds;
        a.host_records = host->records;
        a.host_totals = host->totals;
    }
    if (queue) {
        // The look-back words, ticket counter and accumulators are zero when a
        // launch starts: zeroed once here on (re)allocation, and reset by the
        // last CTA of every launch.  So a batched build is one kernel launch.
        if (!ctx->d_lookback || ctx->lookback_cap < (size_t)n * sizeof(unsigned long long)) {
            st = grow(&ctx->d_lookback, &ctx->lookback_cap, std::max<size_t>((size_t)n, 4096) * sizeof(unsigned long long));
            if (st) return st;
            cudaError_t e = cudaMemsetAsync(ctx->d_lookback, 0, ctx->lookback_cap, ctx->stream);
            if (e != cudaSuccess) return cuda_status(e, "cudaMemsetAsync");
        }
        a.lookback = ctx->d_lookback;
        a.work_counter = ctx->d_counter;
        a.acc = ctx->d_acc;
        // a batch whose samples and cases are neither read nor written is
        // planned: a first kernel lists the chunks the depth bias does not
        // decide, and the build takes only those
        const bool planned = !samples_in && !a.samples_out && !(a.cases && (ctx->params.outputs & UWW_OUT_CASES)) &&
                             !a.no_depth_shortcut;
        if (planned) {
            // its finish counter is zero between launches: cleared here on
            // (re)allocation, re-armed by the planning kernel's last CTA
            if (!ctx->d_plan || ctx->plan_cap < plan_buffer_bytes(n)) {
                st = grow(&ctx->d_plan, &ctx->plan_cap, plan_buffer_bytes(std::max<uint32_t>(n, 4096)));
                if (st) return st;
                cudaError_t e = cudaMemsetAsync(ctx->d_plan, 0, ctx->plan_cap, ctx->stream);
                if (e != cudaSuccess) return cuda_status(e, "cudaMemsetAsync");
            }
            a.plan = ctx->d_plan;
        }
        if (cfg.split) {
            // The counters, the tile sums, per chunk its counts word and its
            // staging place, and the work queues -- laid out for the chunk
            // count the buffer was sized for, so that they stay in place from
            // one launch to the next.  The counters and tile sums are zero at
            // launch: cleared here on (re)allocation and left zero by every
            // launch's emission kernel.  (With slabs: a place per slab for
            // the staging places and the queues.)
            const size_t pm = cfg.pmax;
            auto fixed_bytes = [pm](uint32_t m) {
                const size_t ntiles = ((size_t)m + kTileChunks - 1) / kTileChunks;
                return kCtrWords * 4 + ((ntiles * 8 + 15) & ~size_t(15)) + (((size_t)m * 8 + 15) & ~size_t(15)) +
                       (((size_t)m * pm * 8 + 15) & ~size_t(15)) + (((size_t)m * pm * 4 * kPlanRanks + 15) & ~size_t(15));
            };
            const uint32_t m = std::max(n, ctx->split_n);
            if (!ctx->d_split || ctx->split_n < n || ctx->split_cap < fixed_bytes(m)) {
                const uint32_t mm = std::max(m, 4096u);
                st = grow(&ctx->d_split, &ctx->split_cap, fixed_bytes(mm));
                if (st) return st;
                ctx->split_n = mm;
                const size_t ntiles = ((size_t)mm + kTileChunks - 1) / kTileChunks;
                cudaError_t e = cudaMemsetAsync(ctx->d_split, 0, kCtrWords * 4 + ntiles * 8, ctx->stream);
                if (e != cudaSuccess) return cuda_status(e, "cudaMemsetAsync");
            }
            const uint32_t nc = ctx->split_n;
            const size_t ntiles = ((size_t)nc + kTileChunks - 1) / kTileChunks;
            uint8_t* b = ctx->d_split;
            a.split_ctr = reinterpret_cast<uint32_t*>(b);
            a.stage_ctr = reinterpret_cast<unsigned long long*>(b + kCtrStage * 4);
            b += kCtrWords * 4;
            a.tile_sum = reinterpret_cast<unsigned long long*>(b);
            b += (ntiles * 8 + 15) & ~size_t(15);
            a.tinfo = reinterpret_cast<unsigned long long*>(b);
            b += ((size_t)nc * 8 + 15) & ~size_t(15);
            a.stage_at = reinterpret_cast<unsigned long long*>(b);
            b += ((size_t)nc * pm * 8 + 15) & ~size_t(15);
            a.split_queue = reinterpret_cast<uint32_t*>(b);
            b += ((size_t)nc * pm * 4 * kPlanRanks + 15) & ~size_t(15);
            a.split = 1;
            a.pmax = (uint32_t)pm;
            a.piece_cells = 16;
            if (pm > 1) {
                // per place its counts and its seam (rewritten by every launch)
                const size_t pinfo_bytes = ((size_t)n * pm * 8 + 15) & ~size_t(15);
                a.seam_stride = max_cells * max_cells;
                if ((st = grow(&ctx->d_slab, &ctx->slab_cap, pinfo_bytes + (size_t)n * pm * a.seam_stride * 4)))
                    return st;
                a.pinfo = reinterpret_cast<unsigned long long*>(ctx->d_slab);
                a.seam = reinterpret_cast<uint32_t*>(ctx->d_slab + pinfo_bytes);
            }
            // the emission CTAs' scratch slots, for chunks and slabs built
            // again (their output found no staging room)
            int egrid = 0;
            size_t edyn = 0;
            cudaError_t e = split_emit_shape(ctx->dev, a, &egrid, &edyn);
            if (e != cudaSuccess) return cuda_status(e);
            const size_t eslot = std::max(cfg.slab_slot, (size_t)align16(chunk_layout((int)cfg.smem_cells).total));
            if ((st = grow(&ctx->d_scratch, &ctx->scratch_cap, eslot * (size_t)egrid))) return st;
            a.scratch = ctx->d_scratch;
            a.scratch_slot_bytes = eslot;
            // staging as large as the outputs (a batch whose output fits its
            // capacities is always staged whole), and the emission units:
            // at most one vertex block per kVertexBlock vertices plus one per
            // chunk, one index block per kIndexBlock indices plus one per
            // chunk, one whole chunk per chunk
            const size_t vc = out->vert_capacity, ic = out->ind_capacity;
            const size_t units = vc / kVertexBlock + ic / kIndexBlock + 3 * (size_t)nc * pm;
            const size_t sbytes = vc * 16 + ((ic * 4 + 15) & ~size_t(15)) + units * 8 + (edge_ids ? vc * 4 : 0);
            if (!ctx->d_stage || ctx->stage_cap < sbytes) {
                st = grow(&ctx->d_stage, &ctx->stage_cap, sbytes);
                if (st) return st;
            }
            uint8_t* sb = ctx->d_stage;
            a.stage_pos = reinterpret_cast<float4*>(sb);
            sb += vc * 16;
            a.stage_inds = reinterpret_cast<uint32_t*>(sb);
            sb += (ic * 4 + 15) & ~size_t(15);
            a.units = reinterpret_cast<unsigned long long*>(sb);
            sb += units * 8;
            a.stage_eids = edge_ids ? reinterpret_cast<uint32_t*>(sb) : nullptr;
            a.unit_cap = (uint32_t)std::min<size_t>(units, 0xffffffffu);
            a.stage_vcap = out->vert_capacity;
            a.stage_icap = out->ind_capacity;
            // (a batch with slabs always runs the planning kernel, which
            // queues the slabs; it decides chunks only when planned)
            a.split_planned = a.plan != nullptr || pm > 1;
            a.split_decide = a.plan != nullptr;
            a.plan = nullptr;  // the split build plans into its own queues
        }
    }
    if (prepare_only) return UWW_OK;
    return cuda_status(launch_build(ctx->dev, a, queue, cfg.grid, cfg.threads, cfg.dyn_smem, ctx->stream), "build kernel launch");
}

// The device address of page-locked host memory, or NULL when `p` is not
// host memory the device can address.
void* device_view(void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return at.devicePointer;
}

// device: the buffers are device memory the kernels write (alignment checked);
// otherwise host buffers, reached by copies of any alignment
int check_out(const uww_mesh_out* out, bool device = true)
{
    if (!out || !out->verts || !out->inds || !out->records) return UWW_ERR_INVALID_ARG;
    if (out->vert_capacity > kLbVertMax) return UWW_ERR_INVALID_ARG;
    if (device && !device_out_aligned(out)) return UWW_ERR_INVALID_ARG;
    return UWW_OK;
}

}  // namespace

namespace uww {
int check_params(const uww_params* p) { return validate_params(p); }
void dev_params_from(const uww_params* p, DevParams* d) { make_dev_params(p, d); }
int status_from_cuda(cudaError_t e, const char* where) { return cuda_status(e, where); }
long long spin_limit_cycles() { return kSpinLimitCycles; }
int default_compute_threads(uint32_t max_cells) { return max_cells <= 12 ? 192 : max_cells <= 16 ? 256 : 512; }
int ensure_device_bytes(void** ptr, size_t* cap, size_t bytes) { return ensure_device(ptr, cap, bytes); }
int launch_batched(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                   const uww_mesh_out* out, uint32_t* edge_ids, const uint32_t* n_dev)
{
    return launch(ctx, d_chunks, n, max_cells, out, true, nullptr, 0, edge_ids, n_dev);
}
int check_mesh_out(const uww_mesh_out* out) { return check_out(out); }
int prepare_batched(uww_ctx* ctx, uint32_t n, uint32_t max_cells, const uww_mesh_out* out)
{
    return launch(ctx, nullptr, n, max_cells, out, true, nullptr, 0, nullptr, nullptr, true);
}
int plan_batched(uww_ctx* ctx, uint32_t n, uint32_t max_cells, int* threads, int* grid, size_t* dyn_smem,
                 int* occupancy, uint32_t* split, uint32_t* pmax)
{
    LaunchCfg cfg;
    const int st = plan_launch(ctx, n, max_cells, true, &cfg, true, plans(ctx, nullptr, nullptr));
    if (st) return st;
    *threads = cfg.threads;
    *grid = cfg.grid;
    *dyn_smem = cfg.dyn_smem;
    *occupancy = cfg.occupancy;
    if (split) *split = cfg.split ? 1u : 0u;
    if (pmax) *pmax = cfg.split ? cfg.pmax : 1u;
    return UWW_OK;
}
}  // namespace uww

#pragma GCC visibility push(default)
extern "C" {

int uww_abi_version(void) { return UWW_ABI_VERSION; }

const char* uww_last_error(void) { return g_last_error; }

const char* uww_status_string(int s)
{
    switch (s) {
    case UWW_OK: return "ok";
    case UWW_ERR_INVALID_ARG: return "invalid argument";
    case UWW_ERR_CUDA: return "CUDA error";
    case UWW_ERR_CAPACITY: return "output capacity exceeded";
    case UWW_ERR_OOM: return "out of memory";
    case UWW_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

void uww_params_reference(uww_params* p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->seed = 0;
    p->octaves = 3;             // PERLIN_OCTAVES (chunk.rs:9)
    p->chunk_size = 16;         // CHUNK_SIZE (chunk.rs:5)
    p->base_freq = 1.0f / 16.0f;  // (local + offset) / CHUNK_SIZE (chunk.rs:108)
    p->lacunarity = 2.0f;       // perlin_util.rs:19
    p->persistence = 0.5f;      // perlin_util.rs:18
    p->amplitude = 1.0f;        // perlin_util.rs:9
    p->normalize = 1;           // perlin_util.rs:21
    p->bias_mode = UWW_BIAS_TERRACED;
    p->bias_a = 16.0f;          // CHUNK_SIZE
    p->bias_b = 32.0f;          // MAX_HEIGHT (chunk.rs:11)
    p->bias_c = 0.25f;          // ADJ_Z_MOD (chunk.rs:12)
    p->iso_level = -0.1f;       // ISO_LEVEL (chunk.rs:10)
    p->math_mode = UWW_MATH_EXACT;
    p->dedup_mode = UWW_DEDUP_ORIENTED;
    p->outputs = UWW_OUT_COLOR;
    p->color_min_z = -2.0f;     // world::MIN_Z (world.rs:12)
    p->color_max_z = 2.0f;      // world::MAX_Z (world.rs:11)
}

int uww_perm_table(uint32_t seed, uint8_t out[256])
{
    if (!out) return UWW_ERR_INVALID_ARG;
    make_perm(seed, out);
    return UWW_OK;
}

int uww_layout_cells(uww_chunk_desc* desc, uint32_t n, uint64_t* total_cells, uint64_t* total_samples)
{
    if (!desc && n) return UWW_ERR_INVALID_ARG;
    uint64_t off = 0, soff = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint64_t c = desc[i].cells;
        if (c < 1 || c > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
        if (off > 0xffffffffull || soff > 0xffffffffull) return UWW_ERR_INVALID_ARG;
        desc[i].cell_offset = (uint32_t)off;
        desc[i].sample_offset = (uint32_t)soff;
        off += c * c * c;
        soff += (c + 1) * (c + 1) * (c + 1);
    }
    if (total_cells) *total_cells = off;
    if (total_samples) *total_samples = soff;
    return UWW_OK;
}

int uww_ctx_create(const uww_params* p, void* stream, uww_ctx** out)
{
    if (!out) return UWW_ERR_INVALID_ARG;
    *out = nullptr;
    int st = validate_params(p);
    if (st) return st;
    uww_ctx* ctx = new (std::nothrow) uww_ctx();
    if (!ctx) return UWW_ERR_OOM;
    ctx->params = *p;
    make_dev_params(p, &ctx->dev);
    const char* where = "cudaGetDevice";
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    int optin = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    ctx->smem_optin = (size_t)optin;
    if (e == cudaSuccess) {
        where = "cudaFuncSetAttribute(MaxDynamicSharedMemorySize)";
        e = prepare_build_kernels(ctx->smem_optin, &ctx->smem_dyn_max);
    }
    if (e == cudaSuccess) {
        where = "cudaStreamCreate";
        if (stream) ctx->stream = (cudaStream_t)stream;
        else { e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking); ctx->own_stream = true; }
    }
    if (e == cudaSuccess) {
        where = "cudaMalloc";
        // [0] ticket counter (u32), [1..3] overflow count, error flags, exit count
        e = cudaMalloc((void**)&ctx->d_state, 4 * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMemset(ctx->d_state, 0, 4 * sizeof(unsigned long long));
        ctx->d_counter = reinterpret_cast<unsigned int*>(ctx->d_state);
        ctx->d_acc = ctx->d_state + 1;
    }
    if (e == cudaSuccess) e = cudaMalloc((void**)&ctx->d_totals, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_tables, table_image_bytes());
    if (e == cudaSuccess) { where = "table image"; e = launch_table_image(ctx->dev, ctx->d_tables, ctx->stream); }
    if (e == cudaSuccess) { where = "cudaMallocHost"; e = cudaMallocHost((void**)&ctx->h_totals, 4 * sizeof(unsigned long long)); }
    if (e != cudaSuccess) {
        const int st2 = cuda_status(e, where);
        uww_ctx_destroy(ctx);
        return st2;
    }
    *out = ctx;
    return UWW_OK;
}

int uww_ctx_destroy(uww_ctx* ctx)
{
    if (!ctx) return UWW_ERR_INVALID_ARG;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_lookback);
    cudaFree(ctx->d_plan);
    cudaFree(ctx->d_tables);
    cudaFree(ctx->d_split);
    cudaFree(ctx->d_stage);
    cudaFree(ctx->d_slab);
    cudaFree(ctx->d_state);
    cudaFree(ctx->d_totals);
    cudaFree(ctx->d_scratch);
    cudaFree(ctx->d_chunks);
    cudaFree(ctx->d_verts);
    cudaFree(ctx->d_normals);
    cudaFree(ctx->d_inds);
    cudaFree(ctx->d_cases);
    cudaFree(ctx->d_samples);
    cudaFree(ctx->d_records);
    cudaFree(ctx->d_adj_part);
    cudaFree(ctx->d_adj_counter);
    cudaFree(ctx->d_sample_err);
    if (ctx->h_totals) cudaFreeHost(ctx->h_totals);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return UWW_OK;
}

int uww_ctx_set_params(uww_ctx* ctx, const uww_params* p)
{
    if (!ctx) return UWW_ERR_INVALID_ARG;
    int st = validate_params(p);
    if (st) return st;
    ctx->params = *p;
    make_dev_params(p, &ctx->dev);
    return UWW_OK;
}

int uww_ctx_get_params(const uww_ctx* ctx, uww_params* p)
{
    if (!ctx || !p) return UWW_ERR_INVALID_ARG;
    *p = ctx->params;
    return UWW_OK;
}

void* uww_ctx_stream(uww_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int uww_ctx_sync(uww_ctx* ctx)
{
    if (!ctx) return UWW_ERR_INVALID_ARG;
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int uww_build_chunks(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                     const uww_mesh_out* out)
{
    if (!ctx) return UWW_ERR_INVALID_ARG;
    int st = check_out(out);
    if (st) return st;
    if (max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    if (n == 0) {
        if (out->totals) return cuda_status(cudaMemsetAsync(out->totals, 0, 4 * sizeof(uint64_t), ctx->stream));
        return UWW_OK;
    }
    if (!d_chunks || !aligned_to(d_chunks, 4)) return UWW_ERR_INVALID_ARG;
    return launch(ctx, d_chunks, n, max_cells, out, true);
}

int uww_build_chunks_from_samples(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                                  const float* d_samples, uint64_t sample_count, const uww_mesh_out* out)
{
    if (!ctx) return UWW_ERR_INVALID_ARG;
    int st = check_out(out);
    if (st) return st;
    if (max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    if (n == 0) {
        if (out->totals) return cuda_status(cudaMemsetAsync(out->totals, 0, 4 * sizeof(uint64_t), ctx->stream));
        return UWW_OK;
    }
    if (!d_chunks || !d_samples || !aligned_to(d_chunks, 4) || !aligned_to(d_samples, 4)) return UWW_ERR_INVALID_ARG;
    return launch(ctx, d_chunks, n, max_cells, out, true, d_samples, sample_count);
}

int uww_build_chunk_plain(uww_ctx* ctx, const uww_chunk_desc* d_chunk, uint32_t cells, const uww_mesh_out* out)
{
    if (!ctx || !d_chunk || !aligned_to(d_chunk, 4)) return UWW_ERR_INVALID_ARG;
    int st = check_out(out);
    if (st) return st;
    if (!out->totals) return UWW_ERR_INVALID_ARG;
    if (cells < 1 || cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    return launch(ctx, d_chunk, 1, cells, out, false);
}

int uww_build_chunks_host(uww_ctx* ctx, const uww_chunk_desc* h_chunks, uint32_t n, const uww_mesh_out* h_out)
{
    if (!ctx) return UWW_ERR_INVALID_ARG;
    int st = check_out(h_out, false);
    if (st) return st;
    if (n && !h_chunks) return UWW_ERR_INVALID_ARG;
    const bool want_cases = (ctx->params.outputs & UWW_OUT_CASES) && h_out->cases;
    const bool want_normals = (ctx->params.outputs & UWW_OUT_NORMALS) && h_out->normals;
    const bool want_samples = (ctx->params.outputs & UWW_OUT_SAMPLES) && h_out->samples;
    uint32_t max_cells = 1;
    uint64_t case_bytes = 0, sample_count = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t c = h_chunks[i].cells;
        if (c < 1 || c > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
        max_cells = std::max(max_cells, c);
        case_bytes = std::max<uint64_t>(case_bytes, (uint64_t)h_chunks[i].cell_offset + (uint64_t)c * c * c);
        sample_count = std::max<uint64_t>(sample_count,
                                          (uint64_t)h_chunks[i].sample_offset + (uint64_t)(c + 1) * (c + 1) * (c + 1));
    }
    if (n == 0) {
        if (h_out->totals) std::memset(h_out->totals, 0, 4 * sizeof(uint64_t));
        return UWW_OK;
    }
    cudaStream_t s = ctx->stream;
    if ((st = ensure_device(&ctx->d_chunks, &ctx->chunks_cap, (size_t)n * sizeof(uww_chunk_desc)))) return st;
    if ((st = ensure_device(&ctx->d_records, &ctx->records_cap, (size_t)n * sizeof(uww_chunk_record)))) return st;
    if ((st = ensure_device(&ctx->d_verts, &ctx->verts_cap, (size_t)h_out->vert_capacity * sizeof(uww_vert_color)))) return st;
    if ((st = ensure_device(&ctx->d_inds, &ctx->inds_cap, (size_t)h_out->ind_capacity * sizeof(uint32_t)))) return st;
    if (want_normals && (st = ensure_device(&ctx->d_normals, &ctx->normals_cap, (size_t)h_out->vert_capacity * 12))) return st;
    if (want_cases && (st = ensure_device(&ctx->d_cases, &ctx->cases_cap, (size_t)case_bytes))) return st;
    if (want_samples && (st = ensure_device(&ctx->d_samples, &ctx->samples_cap, (size_t)sample_count * 4))) return st;

    cudaError_t e = cudaMemcpyAsync(ctx->d_chunks, h_chunks, (size_t)n * sizeof(uww_chunk_desc), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_status(e);
    uww_mesh_out d_out;
    d_out.verts = (uww_vert_color*)ctx->d_verts;
    d_out.normals = want_normals ? (float*)ctx->d_normals : nullptr;
    d_out.inds = (uint32_t*)ctx->d_inds;
    d_out.cases = want_cases ? (uint8_t*)ctx->d_cases : nullptr;
    d_out.samples = want_samples ? (float*)ctx->d_samples : nullptr;
    d_out.case_capacity = want_cases ? case_bytes : 0;
    d_out.sample_capacity = want_samples ? sample_count : 0;
    d_out.records = (uww_chunk_record*)ctx->d_records;
    d_out.totals = reinterpret_cast<uint64_t*>(ctx->d_totals);
    d_out.vert_capacity = h_out->vert_capacity;
    d_out.ind_capacity = h_out->ind_capacity;

    // Page-locked host buffers the device can address: the build streams
    // records, indices, vertices and normals into them as chunks finish (the
    // transfer overlaps the build), a copy kernel adds cases and samples, and
    // the host synchronises once.  Otherwise the copies are sized on the host
    // after a first synchronisation.
    void* dv = device_view(h_out->verts);
    void* dn = want_normals ? device_view(h_out->normals) : nullptr;
    void* di = device_view(h_out->inds);
    void* dr = device_view(h_out->records);
    void* dc = want_cases ? device_view(h_out->cases) : nullptr;
    void* ds = want_samples ? device_view(h_out->samples) : nullptr;
    // (the streamed words are 4-byte stores: host buffers off a 4-byte boundary take the copy path)
    const bool words_ok = aligned_to(dv, 4) && aligned_to(dn, 4) && aligned_to(di, 4) && aligned_to(dr, 4);
    const bool mapped = dv && di && dr && (!want_normals || dn) && (!want_cases || dc) && (!want_samples || ds);
    LaunchCfg probe;
    if (mapped && plan_launch(ctx, n, max_cells, true, &probe, true, plans(ctx, &d_out, nullptr)) == UWW_OK &&
        probe.split) {
        // The split build.  Its emission kernel is the only one that writes
        // vertices, normals and indices, each once and in place: with host
        // buffers aligned for its stores (8 bytes for vertices) it stores
        // them straight into them, so the host link carries the output
        // while the emission runs.  Then one copy kernel moves the rest
        // (records, totals; otherwise every output, the vertex, normal and
        // index spans sized from the device totals): no host round trip in
        // between.
        const bool direct = aligned_to(dv, 8) && aligned_to(dn, 4) && aligned_to(di, 4);
        uww_mesh_out o = d_out;
        if (direct) {
            o.verts = static_cast<uww_vert_color*>(dv);
            o.normals = want_normals ? static_cast<float*>(dn) : nullptr;
            o.inds = static_cast<uint32_t*>(di);
        }
        if ((st = launch(ctx, ctx->d_chunks, n, max_cells, &o, true))) return st;
        CopyOut c;
        std::memset(&c, 0, sizeof(c));
        auto seg = [&](const void* src, void* dst, unsigned long long fixed, int count_idx, uint32_t elem,
                       unsigned long long cap) {
            CopySeg& g = c.seg[c.nseg++];
            g.src = static_cast<const uint8_t*>(src);
            g.dst = static_cast<uint8_t*>(dst);
            g.fixed_bytes = fixed;
            g.count_idx = count_idx;
            g.elem_bytes = elem;
            g.cap_elems = cap;
        };
        seg(ctx->d_records, dr, (unsigned long long)n * sizeof(uww_chunk_record), -1, 0, 0);
        if (!direct) {
            seg(ctx->d_verts, dv, 0, 0, (uint32_t)sizeof(uww_vert_color), h_out->vert_capacity);
            if (want_normals) seg(ctx->d_normals, dn, 0, 0, 12u, h_out->vert_capacity);
            seg(ctx->d_inds, di, 0, 1, 4u, h_out->ind_capacity);
        }
        if (want_cases && case_bytes) seg(ctx->d_cases, dc, case_bytes, -1, 0, 0);
        if (want_samples && sample_count) seg(ctx->d_samples, ds, sample_count * 4, -1, 0, 0);
        void* dt = device_view(ctx->h_totals);
        if (dt) seg(ctx->d_totals, dt, 4 * sizeof(unsigned long long), -1, 0, 0);
        if ((e = launch_copy_out(c, ctx->d_totals, ctx->num_sms * 2, s)) != cudaSuccess) return cuda_status(e);
        if (!dt &&
            (e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_status(e);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
        if (h_out->totals) std::memcpy(h_out->totals, ctx->h_totals, 4 * sizeof(uint64_t));
        if (ctx->h_totals[3] & kErrTimeout) return UWW_ERR_TIMEOUT;
        if (ctx->h_totals[3] & (kErrBadChunk | kErrRange)) return UWW_ERR_INVALID_ARG;
        if (ctx->h_totals[2]) return UWW_ERR_CAPACITY;
        return UWW_OK;
    }
    if (mapped && words_ok) {
        HostOut ho;
        ho.verts = static_cast<uww_vert_color*>(dv);
        ho.normals = static_cast<float*>(dn);
        ho.inds = static_cast<uint32_t*>(di);
        ho.records = static_cast<uww_chunk_record*>(dr);
        ho.totals = static_cast<unsigned long long*>(device_view(ctx->h_totals));
        if ((st = launch(ctx, ctx->d_chunks, n, max_cells, &d_out, true, nullptr, 0, nullptr, nullptr, false, &ho)))
            return st;
        CopyOut c;
        std::memset(&c, 0, sizeof(c));
        auto seg = [&](const void* src, void* dst, unsigned long long fixed) {
            CopySeg& g = c.seg[c.nseg++];
            g.src = static_cast<const uint8_t*>(src);
            g.dst = static_cast<uint8_t*>(dst);
            g.fixed_bytes = fixed;
            g.count_idx = -1;
            g.elem_bytes = 0;
            g.cap_elems = 0;
        };
        if (want_cases && case_bytes) seg(ctx->d_cases, dc, case_bytes);
        if (want_samples && sample_count) seg(ctx->d_samples, ds, sample_count * 4);
        if ((e = launch_copy_out(c, ctx->d_totals, ctx->num_sms * 2, s)) != cudaSuccess) return cuda_status(e);
        if (!ho.totals &&
            (e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_status(e);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
        if (h_out->totals) std::memcpy(h_out->totals, ctx->h_totals, 4 * sizeof(uint64_t));
        if (ctx->h_totals[3] & kErrTimeout) return UWW_ERR_TIMEOUT;
        if (ctx->h_totals[3] & (kErrBadChunk | kErrRange)) return UWW_ERR_INVALID_ARG;
        if (ctx->h_totals[2]) return UWW_ERR_CAPACITY;
        return UWW_OK;
    }

    if ((st = launch(ctx, ctx->d_chunks, n, max_cells, &d_out, true))) return st;
    if ((e = cudaMemcpyAsync(h_out->records, ctx->d_records, (size_t)n * sizeof(uww_chunk_record), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    if ((e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
    const uint64_t tv = std::min<uint64_t>(ctx->h_totals[0], h_out->vert_capacity);
    const uint64_t ti = std::min<uint64_t>(ctx->h_totals[1], h_out->ind_capacity);
    if (tv && (e = cudaMemcpyAsync(h_out->verts, ctx->d_verts, tv * sizeof(uww_vert_color), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    if (tv && want_normals && (e = cudaMemcpyAsync(h_out->normals, ctx->d_normals, tv * 12, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    if (ti && (e = cudaMemcpyAsync(h_out->inds, ctx->d_inds, ti * sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    if (want_cases && case_bytes && (e = cudaMemcpyAsync(h_out->cases, ctx->d_cases, case_bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    if (want_samples && sample_count &&
        (e = cudaMemcpyAsync(h_out->samples, ctx->d_samples, sample_count * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
    if (h_out->totals) std::memcpy(h_out->totals, ctx->h_totals, 4 * sizeof(uint64_t));
    if (ctx->h_totals[3] & kErrTimeout) return UWW_ERR_TIMEOUT;
    if (ctx->h_totals[3] & (kErrBadChunk | kErrRange)) return UWW_ERR_INVALID_ARG;
    if (ctx->h_totals[2]) return UWW_ERR_CAPACITY;
    return UWW_OK;
}

int uww_ctx_set_tuning(uww_ctx* ctx, const uww_tuning* t)
{
    if (!ctx || !t) return UWW_ERR_INVALID_ARG;
    if (t->threads < 0 || t->threads > 512 || (t->threads % 32) != 0) return UWW_ERR_INVALID_ARG;
    if (t->threads > 192 && t->threads < 224) return UWW_ERR_INVALID_ARG;  // between the two kernel shapes
    if (t->blocks_per_sm < 0 || t->blocks_per_sm > 32) return UWW_ERR_INVALID_ARG;
    if (t->smem_cells < 0 || t->smem_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    if (t->spin_limit < 0 || (t->test_flags & ~(UWW_TEST_WITHHOLD_FIRST | UWW_TEST_WITHHOLD_RECORDS)))
        return UWW_ERR_INVALID_ARG;
    if (t->options & ~(UWW_TUNE_NO_DEPTH_SHORTCUT | UWW_TUNE_PIPELINED)) return UWW_ERR_INVALID_ARG;
    ctx->threads = t->threads;
    ctx->blocks_per_sm = t->blocks_per_sm;
    ctx->smem_cells = t->smem_cells;
    ctx->spin_limit = t->spin_limit;
    ctx->test_flags = t->test_flags;
    ctx->options = t->options;
    return UWW_OK;
}

int uww_ctx_get_tuning(const uww_ctx* ctx, uww_tuning* t)
{
    if (!ctx || !t) return UWW_ERR_INVALID_ARG;
    t->threads = ctx->threads;
    t->blocks_per_sm = ctx->blocks_per_sm;
    t->smem_cells = ctx->smem_cells;
    t->spin_limit = (int32_t)ctx->spin_limit;
    t->test_flags = ctx->test_flags;
    t->options = ctx->options;
    t->reserved[0] = t->reserved[1] = 0;
    return UWW_OK;
}

int uww_launch_shape_of(uww_ctx* ctx, uint32_t n, uint32_t max_cells, uww_launch_shape* out)
{
    if (!ctx || !out || n == 0 || max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    int threads = 0, grid = 0, occ = 0;
    size_t dyn = 0;
    uint32_t split = 0, pmax = 1;
    const int st = plan_batched(ctx, n, max_cells, &threads, &grid, &dyn, &occ, &split, &pmax);
    if (st) return st;
    out->build = split ? UWW_BUILD_SPLIT : UWW_BUILD_PIPELINED;
    out->slabs_per_chunk = pmax;
    out->threads = (uint32_t)threads;
    out->grid = (uint32_t)grid;
    out->blocks_per_sm = (uint32_t)(ctx->blocks_per_sm > 0 ? ctx->blocks_per_sm : occ);
    out->dyn_smem = (uint32_t)dyn;
    return UWW_OK;
}

int uww_device_alloc(size_t bytes, void** out)
{
    if (!out) return UWW_ERR_INVALID_ARG;
    *out = nullptr;
    return cuda_status(cudaMalloc(out, bytes ? bytes : 1));
}

int uww_device_free(void* p) { return cuda_status(cudaFree(p)); }

int uww_host_alloc(size_t bytes, void** out)
{
    if (!out) return UWW_ERR_INVALID_ARG;
    *out = nullptr;
    return cuda_status(cudaMallocHost(out, bytes ? bytes : 1));
}

int uww_host_free(void* p) { return cuda_status(cudaFreeHost(p)); }

int uww_memcpy(uww_ctx* ctx, void* dst, const void* src, size_t bytes, int kind)
{
    if (!ctx || (bytes && (!dst || !src))) return UWW_ERR_INVALID_ARG;
    cudaMemcpyKind k;
    switch (kind) {
    case 0: k = cudaMemcpyHostToDevice; break;
    case 1: k = cudaMemcpyDeviceToHost; break;
    case 2: k = cudaMemcpyDeviceToDevice; break;
    default: return UWW_ERR_INVALID_ARG;
    }
    if (!bytes) return UWW_OK;
    return cuda_status(cudaMemcpyAsync(dst, src, bytes, k, ctx->stream));
}

int uww_memset(uww_ctx* ctx, void* dst, int value, size_t bytes)
{
    if (!ctx || (bytes && !dst)) return UWW_ERR_INVALID_ARG;
    if (!bytes) return UWW_OK;
    return cuda_status(cudaMemsetAsync(dst, value, bytes, ctx->stream));
}

int uww_density_at(uww_ctx* ctx, const float* d_xyz, uint32_t n, float* d_out)
{
    if (!ctx || (n && (!d_xyz || !d_out))) return UWW_ERR_INVALID_ARG;
    return cuda_status(launch_density(ctx->dev, d_xyz, n, d_out, ctx->stream));
}

}  // extern "C"
#pragma GCC visibility pop
