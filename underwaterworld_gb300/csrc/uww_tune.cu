// uww_tune.cu -- the per-frame build as a CUDA graph, and the autotuner.
//
// The reference builds a few chunks per frame on the CPU (world.rs:113-145,
// Chunk::build_partial, chunk.rs:270-290).  Here a frame's whole chunk list
// is one graph launch: descriptor and count upload, the persistent batched
// build (which reads its chunk count from device memory, so one graph serves
// any count up to its maximum), and the download of records and totals.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "uww_internal.h"

using namespace uww;

struct uww_frame {
    uww_ctx* ctx = nullptr;
    uint32_t max_chunks = 0;
    uint32_t max_cells = 0;
    const uww_chunk_desc* h_chunks = nullptr;
    const uint32_t* h_count = nullptr;
    uww_chunk_record* h_records = nullptr;
    uint64_t* h_totals = nullptr;
    uww_mesh_out out{};
    uww_chunk_desc* d_chunks = nullptr;
    uint32_t* d_count = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t gen = 0;  // the context's work-buffer generation the graph was captured with
};

namespace {

// Record the frame's work on the context stream into a new graph.
int capture_frame(uww_frame* f, cudaGraph_t* out)
{
    uww_ctx* ctx = f->ctx;
    cudaStream_t s = ctx->stream;
    // allocations and their first clearing happen outside the capture
    int st = prepare_batched(ctx, f->max_chunks, f->max_cells, &f->out);
    if (st) return st;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaStreamBeginCapture");
    cudaError_t ce = cudaMemcpyAsync(f->d_chunks, f->h_chunks, (size_t)f->max_chunks * sizeof(uww_chunk_desc),
                                     cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(f->d_count, f->h_count, sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    int lst = ce == cudaSuccess ? launch_batched(ctx, f->d_chunks, f->max_chunks, f->max_cells, &f->out, nullptr, f->d_count)
                                : UWW_ERR_CUDA;
    const void* d_totals = f->out.totals ? (const void*)f->out.totals : (const void*)ctx->d_totals;
    if (lst == UWW_OK && f->h_records)
        ce = cudaMemcpyAsync(f->h_records, f->out.records, (size_t)f->max_chunks * sizeof(uww_chunk_record),
                             cudaMemcpyDeviceToHost, s);
    if (lst == UWW_OK && ce == cudaSuccess && f->h_totals)
        ce = cudaMemcpyAsync(f->h_totals, d_totals, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(s, &g);
    if (ce != cudaSuccess || lst != UWW_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (lst != UWW_OK) return lst;
        return status_from_cuda(ce != cudaSuccess ? ce : e, "frame capture");
    }
    *out = g;
    f->gen = ctx->work_gen;
    return UWW_OK;
}

// Capture the frame again and update the executable graph with it
// (re-instantiated when the launch shape changed).
int recapture_frame(uww_frame* f)
{
    cudaGraph_t g = nullptr;
    int st = capture_frame(f, &g);
    if (st) return st;
    cudaGraphExecUpdateResultInfo info;
    cudaError_t e = cudaGraphExecUpdate(f->exec, g, &info);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaGraphExec_t x = nullptr;
        e = cudaGraphInstantiate(&x, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return status_from_cuda(e, "cudaGraphInstantiate");
        }
        cudaGraphExecDestroy(f->exec);
        f->exec = x;
    }
    cudaGraphDestroy(f->graph);
    f->graph = g;
    return UWW_OK;
}

// ---- autotuner ----------------------------------------------------------------
std::string tune_key(const uww_ctx* ctx, const std::vector<uww_chunk_desc>& h, uint32_t max_cells)
{
    cudaDeviceProp prop;
    std::memset(&prop, 0, sizeof(prop));
    cudaGetDeviceProperties(&prop, ctx->device);
    std::map<uint32_t, size_t> hist;
    for (const auto& d : h) hist[d.cells]++;
    // batch size to a power of two, LOD shares to 5 %
    int lg = 0;
    while ((1ull << (lg + 1)) <= h.size()) ++lg;
    char buf[512];
    int o = std::snprintf(buf, sizeof(buf), "%s|sm%d|n2^%d|max%u|", prop.name, ctx->num_sms, lg, max_cells);
    for (const auto& kv : hist) {
        const int pct = (int)std::lround(20.0 * (double)kv.second / (double)h.size()) * 5;
        o += std::snprintf(buf + o, sizeof(buf) - (size_t)o, "%u:%d,", kv.first, pct);
        if (o >= (int)sizeof(buf) - 64) break;
    }
    const uww_params& p = ctx->params;
    std::snprintf(buf + o, sizeof(buf) - (size_t)o, "|oct%u|out%u|math%d|dedup%d|norm%d|bias%d", p.octaves,
                  p.outputs, p.math_mode, p.dedup_mode, p.normalize, p.bias_mode);
    std::string k(buf);
    for (char& c : k)
        if (c == ' ' || c == '\t' || c == '\n') c = '_';
    return k;
}

bool cache_lookup(const char* path, const std::string& key, uww_tuning* t, float* us)
{
    FILE* fp = std::fopen(path, "r");
    if (!fp) return false;
    char line[1024];
    bool found = false;
    while (std::fgets(line, sizeof(line), fp)) {
        char k[768];
        int th, bps, sc;
        float u;
        if (std::sscanf(line, "%767s %d %d %d %f", k, &th, &bps, &sc, &u) == 5 && key == k) {
            t->threads = th;
            t->blocks_per_sm = bps;
            t->smem_cells = sc;
            *us = u;
            found = true;  // the last entry for a key wins
        }
    }
    std::fclose(fp);
    return found;
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

int uww_frame_create(uww_ctx* ctx, uint32_t max_chunks, uint32_t max_cells, const uww_chunk_desc* h_chunks,
                     const uint32_t* h_count, const uww_mesh_out* d_out, uww_chunk_record* h_records,
                     uint64_t* h_totals, uww_frame** out)
{
    if (!out) return UWW_ERR_INVALID_ARG;
    *out = nullptr;
    if (!ctx || !h_chunks || !h_count || max_chunks == 0) return UWW_ERR_INVALID_ARG;
    if (max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    int st = check_mesh_out(d_out);
    if (st) return st;
    uww_frame* f = new (std::nothrow) uww_frame();
    if (!f) return UWW_ERR_OOM;
    f->ctx = ctx;
    f->max_chunks = max_chunks;
    f->max_cells = max_cells;
    f->h_chunks = h_chunks;
    f->h_count = h_count;
    f->h_records = h_records;
    f->h_totals = h_totals;
    f->out = *d_out;
    cudaError_t e = cudaMalloc((void**)&f->d_chunks, (size_t)max_chunks * sizeof(uww_chunk_desc));
    if (e == cudaSuccess) e = cudaMalloc((void**)&f->d_count, sizeof(uint32_t));
    if (e != cudaSuccess) {
        st = status_from_cuda(e, "cudaMalloc");
        uww_frame_destroy(f);
        return st;
    }
    st = capture_frame(f, &f->graph);
    if (st == UWW_OK) {
        e = cudaGraphInstantiate(&f->exec, f->graph, 0);
        if (e != cudaSuccess) st = status_from_cuda(e, "cudaGraphInstantiate");
    }
    if (st != UWW_OK) {
        uww_frame_destroy(f);
        return st;
    }
    *out = f;
    return UWW_OK;
}

int uww_frame_launch(uww_frame* f)
{
    if (!f || !f->exec) return UWW_ERR_INVALID_ARG;
    if (*f->h_count > f->max_chunks) return UWW_ERR_INVALID_ARG;
    // another build on the context reallocated a work buffer the graph uses
    if (f->gen != f->ctx->work_gen) {
        const int st = recapture_frame(f);
        if (st) return st;
    }
    return status_from_cuda(cudaGraphLaunch(f->exec, f->ctx->stream), "cudaGraphLaunch");
}

int uww_frame_set_params(uww_frame* f, const uww_params* p)
{
    if (!f) return UWW_ERR_INVALID_ARG;
    int st = uww_ctx_set_params(f->ctx, p);
    if (st) return st;
    return recapture_frame(f);
}

int uww_frame_destroy(uww_frame* f)
{
    if (!f) return UWW_ERR_INVALID_ARG;
    if (f->ctx && f->ctx->stream) cudaStreamSynchronize(f->ctx->stream);
    if (f->exec) cudaGraphExecDestroy(f->exec);
    if (f->graph) cudaGraphDestroy(f->graph);
    cudaFree(f->d_chunks);
    cudaFree(f->d_count);
    delete f;
    return UWW_OK;
}

int uww_autotune(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                 const uww_mesh_out* out, const char* cache_path, uww_tuning* best, float* best_us)
{
    if (!ctx || !d_chunks || n == 0 || !best) return UWW_ERR_INVALID_ARG;
    if (max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    int st = check_mesh_out(out);
    if (st) return st;
    cudaStream_t s = ctx->stream;
    std::vector<uww_chunk_desc> h(n);
    cudaError_t e = cudaMemcpyAsync(h.data(), d_chunks, (size_t)n * sizeof(uww_chunk_desc), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return status_from_cuda(e, "autotune descriptor read");
    const std::string key = tune_key(ctx, h, max_cells);
    float us = 0.f;
    uww_ctx_get_tuning(ctx, best);  // a cached entry sets the launch shape; the rest stays the context's
    if (cache_path && cache_lookup(cache_path, key, best, &us)) {
        if (best_us) *best_us = us;
        return uww_ctx_set_tuning(ctx, best);
    }

    // candidates: compute threads per CTA (about one per sample column of a
    // chunk, up to the large-chunk shape), CTAs per SM, and the LOD at which
    // chunks move from shared memory to a global scratch slot
    std::vector<int> threads = {64, 96, 128, 160, 192};
    if (max_cells > 12) for (int t : {256, 320, 384, 448, 512}) threads.push_back(t);
    std::vector<int> smem = {0};
    for (int c : {24, 16, 12})
        if ((uint32_t)c < max_cells) smem.push_back(c);
    uww_tuning saved;
    uww_ctx_get_tuning(ctx, &saved);
    uww_tuning bt = saved;
    float bus = INFINITY;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return status_from_cuda(e, "cudaEventCreate");
    }
    std::vector<uint64_t> tot(4);
    const void* d_totals = out->totals ? (const void*)out->totals : (const void*)ctx->d_totals;
    for (int sc : smem) {
        for (int th : threads) {
            ctx->threads = th;
            ctx->smem_cells = sc;
            ctx->blocks_per_sm = 0;
            int thr = 0, grid = 0;
            size_t dyn = 0;
            int occ = 0;
            if (plan_batched(ctx, n, max_cells, &thr, &grid, &dyn, &occ) || occ < 1) {
                cudaGetLastError();
                continue;
            }
            for (int bps = 1; bps <= occ; ++bps) {
                if (bps > 2 && bps < occ && (bps & 1)) continue;  // 1, 2, even counts and the maximum
                ctx->blocks_per_sm = bps;
                float best_rep = INFINITY;
                bool ok = true;
                for (int rep = 0; rep < 4 && ok; ++rep) {
                    e = cudaEventRecord(e0, s);
                    st = launch_batched(ctx, d_chunks, n, max_cells, out, nullptr, nullptr);
                    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    if (st || e != cudaSuccess) { ok = false; break; }
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) best_rep = std::min(best_rep, ms * 1e3f);  // the first run warms up
                }
                if (!ok) break;
                e = cudaMemcpy(tot.data(), d_totals, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost);
                if (e != cudaSuccess) break;
                if (tot[2] || tot[3]) {
                    st = tot[3] ? UWW_ERR_INVALID_ARG : UWW_ERR_CAPACITY;
                    ok = false;
                }
                if (!ok) break;
                if (best_rep < bus) {
                    bus = best_rep;
                    bt = saved;  // keeps the context's spin limit and test flags
                    bt.threads = th;
                    bt.blocks_per_sm = bps;
                    bt.smem_cells = sc;
                }
            }
            if (st || e != cudaSuccess) break;
        }
        if (st || e != cudaSuccess) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->threads = saved.threads;
    ctx->blocks_per_sm = saved.blocks_per_sm;
    ctx->smem_cells = saved.smem_cells;
    if (e != cudaSuccess) return status_from_cuda(e, "autotune");
    if (st) return st;
    if (!std::isfinite(bus)) return UWW_ERR_INVALID_ARG;
    *best = bt;
    if (best_us) *best_us = bus;
    if (cache_path) {
        FILE* fp = std::fopen(cache_path, "a");
        if (fp) {
            std::fprintf(fp, "%s %d %d %d %.3f\n", key.c_str(), bt.threads, bt.blocks_per_sm, bt.smem_cells, bus);
            std::fclose(fp);
        }
    }
    return uww_ctx_set_tuning(ctx, &bt);
}

}  // extern "C"
#pragma GCC visibility pop
