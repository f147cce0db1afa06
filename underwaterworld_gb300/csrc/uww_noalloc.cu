// uww_noalloc.cu -- the batched chunk build for callers that cannot allocate.
//
// Some callers of the chunk builder cannot call cudaMalloc: an engine whose
// allocator owns all device memory (it hands out pre-sized buffers and
// forbids other allocations), code running where allocation is not allowed
// (a real-time frame callback that must not stall on the driver's allocator),
// or a host that budgets device memory up front.  uww_build_chunks_noalloc
// serves them: the caller passes descriptors and output buffers it already
// owns, and the build's own scratch -- the work-queue counter, the
// accumulators and the look-back words of the device-wide prefix sum -- lives
// in one file-scope __device__ array of fixed size, below.  No context is
// needed (a context allocates), and no cudaMalloc, cudaFree or allocating
// library routine is called.
//
// Limits and rules:
//   * at most kNoAllocMaxChunks chunks per call (the array holds one look-back
//     word per chunk); larger batches are rejected with UWW_ERR_INVALID_ARG;
//   * every chunk's working set must fit in shared memory (the allocating
//     entry point gives larger chunks a global scratch slot; this one has
//     none), which holds for chunks up to about 18 cells per edge -- the
//     reference's 12^3 chunks included; larger ones are rejected;
//   * the array is shared by every call in the process on a device and keeps
//     the last call's contents, so each call clears the part it uses before
//     its launch; calls that overlap on the GPU (different streams, or other
//     threads) race on it and must be serialised by the caller;
//   * every GPU that loads the library holds the array (about 512 KB) until
//     the process exits;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and sets the kernels' shared-memory limit; make
//     that first call before any stream capture.  The result is kept for the
//     life of the process: a cudaDeviceReset() on that device (which creates
//     a new primary context) is not supported afterwards;
//   * out->totals is required: the four totals words are the call's only
//     report of a timed-out wait, a bad descriptor or an output overflow.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "uww_internal.h"

namespace {

constexpr uint32_t kNoAllocMaxChunks = 65536;
// word 0: ticket counter (low 32 bits); 1..3: overflow count, error flags,
// finished CTAs; 4..7: unused; 8..: look-back words
constexpr size_t kHeadWords = 8;
constexpr size_t kScratchWords = kHeadWords + kNoAllocMaxChunks;

// In host code this name is a host-side stand-in, not a device address: the
// device address comes from cudaGetSymbolAddress, per device, in setup().
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;

struct DeviceSetup {
    bool done;
    unsigned long long* scratch;  // device address of g_noalloc_scratch on this device
    size_t smem_dyn_max;
    int num_sms;
};

DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

// Once per device, with that device current.
int setup(int dev, DeviceSetup** out)
{
    if (dev < 0 || dev >= kMaxDevices) return UWW_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& s = g_setup[dev];
    if (!s.done) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return uww::status_from_cuda(e, "cudaGetSymbolAddress");
        int sms = 0, optin = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return uww::status_from_cuda(e, "cudaDeviceGetAttribute");
        size_t dyn = 0;
        e = uww::prepare_build_kernels((size_t)optin, &dyn);
        if (e != cudaSuccess) return uww::status_from_cuda(e, "cudaFuncSetAttribute(MaxDynamicSharedMemorySize)");
        s.scratch = static_cast<unsigned long long*>(ptr);
        s.smem_dyn_max = dyn;
        s.num_sms = sms;
        s.done = true;
    }
    *out = &s;
    return UWW_OK;
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" int uww_build_chunks_noalloc(const uww_params* params, void* stream, const uww_chunk_desc* d_chunks,
                                        uint32_t n, uint32_t max_cells, const uww_mesh_out* out)
{
    using namespace uww;
    int st = check_params(params);
    if (st) return st;
    if (!out || !out->verts || !out->inds || !out->records) return UWW_ERR_INVALID_ARG;
    // without totals a timeout, a bad descriptor or an overflow would go unreported
    if (!out->totals) return UWW_ERR_INVALID_ARG;
    if (out->vert_capacity > kLbVertMax) return UWW_ERR_INVALID_ARG;
    if (!device_out_aligned(out)) return UWW_ERR_INVALID_ARG;
    if (max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    if (n > kNoAllocMaxChunks) return UWW_ERR_INVALID_ARG;  // beyond the fixed scratch
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) return status_from_cuda(cudaMemsetAsync(out->totals, 0, 4 * sizeof(uint64_t), s), "cudaMemsetAsync");
    if (!d_chunks || !aligned_to(d_chunks, 4)) return UWW_ERR_INVALID_ARG;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaGetDevice");
    DeviceSetup* ds = nullptr;
    if ((st = setup(dev, &ds))) return st;

    DevParams dp;
    dev_params_from(params, &dp);

    // two chunk workspaces (the pipelined batch) and the z tables, all in
    // shared memory: chunks that would need a global scratch slot are refused
    const uint32_t slots = 2;
    const size_t buf = chunk_layout((int)max_cells).total;
    const size_t zt = dp.math_mode == UWW_MATH_FAST ? ztable_bytes((int)max_cells + 1, dp.octaves) : 0;
    const size_t dyn = slots * buf + zt;
    if (dyn > ds->smem_dyn_max) return UWW_ERR_INVALID_ARG;
    const int threads = default_compute_threads(max_cells) + 32;
    int bps = 0;
    e = build_occupancy(true, dp.math_mode == UWW_MATH_EXACT, threads, dyn, &bps);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (bps < 1) return UWW_ERR_INVALID_ARG;
    const long long grid = std::min<long long>((long long)bps * ds->num_sms, (long long)n);

    // the array keeps the last call's contents: clear the part this call uses
    unsigned long long* scratch = ds->scratch;
    e = cudaMemsetAsync(scratch, 0, (kHeadWords + n) * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaMemsetAsync");

    BuildArgs a;
    std::memset(&a, 0, sizeof(a));
    a.chunks = d_chunks;
    a.n = n;
    a.max_cells = max_cells;
    a.verts = out->verts;
    a.normals = out->normals;
    a.inds = out->inds;
    a.cases = out->cases;
    a.samples_out = (params->outputs & UWW_OUT_SAMPLES) ? out->samples : nullptr;
    a.samples_in = nullptr;
    a.case_capacity = out->case_capacity;
    a.sample_capacity = out->sample_capacity;
    a.records = out->records;
    a.totals = reinterpret_cast<unsigned long long*>(out->totals);
    a.vert_capacity = out->vert_capacity;
    a.ind_capacity = out->ind_capacity;
    a.lookback = scratch + kHeadWords;
    a.work_counter = reinterpret_cast<unsigned int*>(scratch);
    a.acc = scratch + 1;
    a.scratch = nullptr;
    a.scratch_slot_bytes = 0;
    a.slots_per_cta = slots;
    a.smem_buf_bytes = buf;
    a.ztable_offset = slots * buf;
    a.smem_cells = max_cells;
    a.spin_limit_cycles = spin_limit_cycles();
    return status_from_cuda(launch_build(dp, a, true, (int)grid, threads, dyn, s), "build kernel launch");
}
#pragma GCC visibility pop
