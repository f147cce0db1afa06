/*
 * uww.h -- C ABI of the GB300 chunk-generation library (libuww_gb300.so).
 *
 * It replaces the terrain chunk builder of LelsersLasers/UnderwaterWorld:
 *   - noise::Perlin::new(seed)                      (underwater_world/src/state.rs:359)
 *   - perlin_util::perlin_3d_octaves / iso_at       (underwater_world/src/perlin_util.rs:6-29)
 *   - Chunk::new / build_full / build_partial       (underwater_world/src/chunk.rs:89-103,266-313)
 *     with build_iso, early_blank_check, build_mesh (chunk.rs:105-264)
 *   - Chunk::not_blank / verts_buffer_slice / inds_buffer_slice / num_inds (chunk.rs:344-348)
 *   - draw::VertColor                               (underwater_world/src/draw.rs:4-33)
 *
 * Every call returns an int status (UWW_OK == 0).  Device-pointer calls are
 * asynchronous on the context's stream; the *_host calls copy in, build, copy
 * out and synchronise.  A context is not re-entrant: one host thread at a time.
 * No call falls back to the CPU: without a CUDA device they return
 * UWW_ERR_CUDA.
 */
#ifndef UWW_H
#define UWW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UWW_ABI_VERSION 3

/* ---- status codes --------------------------------------------------------- */
#define UWW_OK               0
#define UWW_ERR_INVALID_ARG  1  /* bad pointer, size, LOD or parameter          */
#define UWW_ERR_CUDA         2  /* CUDA runtime error (no device, launch fault) */
#define UWW_ERR_CAPACITY     3  /* outputs did not fit; counts are valid, grow and rebuild */
#define UWW_ERR_OOM          4  /* device or host allocation failed             */
#define UWW_ERR_TIMEOUT      5  /* a bounded device-side wait gave up           */

/* ---- limits ---------------------------------------------------------------- */
#define UWW_MAX_OCTAVES 16
#define UWW_MAX_CELLS   64      /* cells per chunk edge; 12, 24, 48 are the LODs used */

/* ---- parameter enums ------------------------------------------------------ */
#define UWW_BIAS_NONE      0    /* density = fBm                                       */
#define UWW_BIAS_TERRACED  1    /* iso_at: adj = (nz*a)/b; d = (adj + fBm) - fmod(adj, c)  (perlin_util.rs:24-29) */
#define UWW_BIAS_LINEAR    2    /* d = fBm + a*(world_z - b)                           */

#define UWW_MATH_EXACT 0        /* reference f32 operation order, no FMA contraction (parity build) */
#define UWW_MATH_FAST  1        /* FMA-contracted, table-driven noise (fast build)                  */

#define UWW_DEDUP_ORIENTED 0    /* reference: one vertex per ordered corner pair (chunk.rs:233) */
#define UWW_DEDUP_EDGE     1    /* one vertex per cube edge (both orientations share it)       */

#define UWW_OUT_COLOR    1u     /* VertColor.color (sRGB depth ramp, chunk.rs:212-219)      */
#define UWW_OUT_NORMALS  2u     /* per-vertex unit normal from the analytic density gradient */
#define UWW_OUT_CASES    4u     /* per-cell 8-bit marching-cubes case index                  */
#define UWW_OUT_SAMPLES  8u     /* the (cells+1)^3 f32 density samples (Build::isos, chunk.rs:43) */

/* ---- chunk flags (uww_chunk_record.flags) --------------------------------- */
#define UWW_CHUNK_EARLY_BLANK 1u  /* every sample above the iso-level: early_blank_check (chunk.rs:131-133) */
#define UWW_CHUNK_HAS_MESH    2u  /* num_inds > 0: Chunk::not_blank (chunk.rs:344)                          */
#define UWW_CHUNK_OVERFLOW    4u  /* this chunk's mesh did not fit the output capacity; not written          */

/* World / density parameters.  uww_params_reference() fills the constants of
 * chunk.rs:5-17, perlin_util.rs:6-29 and world.rs:11-12. */
typedef struct uww_params {
    uint32_t seed;          /* permutation seed, noise::Perlin::new(seed) (state.rs:359)        */
    uint32_t octaves;       /* PERLIN_OCTAVES = 3 (chunk.rs:9); 1..UWW_MAX_OCTAVES             */
    int32_t  chunk_size;    /* CHUNK_SIZE = 16 world units per chunk edge (chunk.rs:5)         */
    float    base_freq;     /* noise units per world unit; 1/16 (chunk.rs:108: /CHUNK_SIZE)    */
    float    lacunarity;    /* frequency *= 2.0 (perlin_util.rs:19)                            */
    float    persistence;   /* amplitude *= 0.5 (perlin_util.rs:18)                            */
    float    amplitude;     /* first-octave amplitude, 1.0 (perlin_util.rs:9)                  */
    int32_t  normalize;     /* 1: total / sum(amplitudes) (perlin_util.rs:21)                  */
    int32_t  bias_mode;     /* UWW_BIAS_*                                                      */
    float    bias_a;        /* terraced: CHUNK_SIZE (16); linear: slope per world unit          */
    float    bias_b;        /* terraced: MAX_HEIGHT (32); linear: z0 in world units             */
    float    bias_c;        /* terraced: ADJ_Z_MOD (0.25); linear: unused                       */
    float    iso_level;     /* ISO_LEVEL = -0.1 (chunk.rs:10); case bit i set when d_i < iso   */
    float    offset[3];     /* world-space offset added to the noise input (0 in the reference) */
    int32_t  explicit_amps; /* 1: per-octave amplitudes come from amps[]                       */
    float    amps[UWW_MAX_OCTAVES];
    int32_t  math_mode;     /* UWW_MATH_*                                                      */
    int32_t  dedup_mode;    /* UWW_DEDUP_*                                                     */
    uint32_t outputs;       /* UWW_OUT_* mask                                                  */
    float    color_min_z;   /* world::MIN_Z = -2, in chunks (world.rs:12)                      */
    float    color_max_z;   /* world::MAX_Z =  2, in chunks (world.rs:11)                      */
} uww_params;

/* One chunk to build.  pos is the chunk coordinate (Chunk::new(pos), chunk.rs:89);
 * the chunk covers world [pos*chunk_size, (pos+1)*chunk_size) sampled at
 * (cells+1)^3 points.  cell_offset is where this chunk's per-cell outputs
 * (cases) start and sample_offset where its (cells+1)^3 samples start in a
 * sample-grid array; uww_layout_cells() fills both. */
typedef struct uww_chunk_desc {
    int32_t  pos[3];
    uint32_t cells;         /* 1..UWW_MAX_CELLS; the reference uses INTERNAL_SIZE = 12 */
    uint32_t cell_offset;
    uint32_t sample_offset;
    uint32_t reserved[2];
} uww_chunk_desc;           /* 32 bytes */

/* Per-chunk result. Offsets index the batch's vertex and index arrays; index
 * values are chunk-local vertex ids (as in the reference's per-chunk buffers). */
typedef struct uww_chunk_record {
    uint32_t num_verts;
    uint32_t num_inds;      /* Chunk::num_inds (chunk.rs:348)       */
    uint32_t vert_offset;
    uint32_t ind_offset;
    uint32_t flags;         /* UWW_CHUNK_*                          */
    uint32_t num_active_cells;
    uint32_t reserved[2];
} uww_chunk_record;         /* 32 bytes */

/* draw::VertColor (draw.rs:4-9): #[repr(C)] { pos: [f32;3], color: [f32;3] }, stride 24. */
typedef struct uww_vert_color {
    float pos[3];
    float color[3];
} uww_vert_color;

/* Output buffers of a build.  Device pointers for uww_build_chunks*, host
 * pointers for uww_build_chunks_host.  verts/inds/records are required; the
 * others may be NULL (then that output is skipped even if requested).  Device
 * buffers must be aligned as the kernels store to them -- verts and totals to
 * 8 bytes, normals, inds, records and samples to 4 -- and device descriptors
 * to 4 bytes; anything else is refused with UWW_ERR_INVALID_ARG before a
 * launch.  Host buffers may have any alignment. */
typedef struct uww_mesh_out {
    uww_vert_color*   verts;      /* vert_capacity entries                              */
    float*            normals;    /* 3 * vert_capacity floats, or NULL                  */
    uint32_t*         inds;       /* ind_capacity entries                               */
    uint8_t*          cases;      /* sum(cells^3) bytes at desc.cell_offset, or NULL    */
    float*            samples;    /* (cells+1)^3 f32 per chunk at desc.sample_offset, or NULL */
    uww_chunk_record* records;    /* one per chunk                                      */
    uint64_t*         totals;     /* device/host [4]: verts, inds, overflowed chunks, error flags; or NULL */
    uint32_t          vert_capacity;
    uint32_t          ind_capacity;
    uint64_t          case_capacity;    /* bytes available at cases; a chunk whose cells would
                                           fall outside is not written and raises UWW_ERRFLAG_RANGE */
    uint64_t          sample_capacity;  /* floats available at samples; same rule             */
} uww_mesh_out;

/* totals[3] error flags of a device build */
#define UWW_ERRFLAG_TIMEOUT 1u   /* a bounded device wait gave up (UWW_ERR_TIMEOUT)          */
#define UWW_ERRFLAG_BAD     2u   /* a descriptor had cells outside 1..max_cells, or its
                                    input samples lay outside the given sample array          */
#define UWW_ERRFLAG_RANGE   4u   /* a per-cell or per-sample output lay outside its capacity */

typedef struct uww_ctx uww_ctx;

/* ---- library --------------------------------------------------------------- */
int         uww_abi_version(void);
const char* uww_status_string(int status);
/* Text of the last CUDA error seen by a call on this host thread ("" if none). */
const char* uww_last_error(void);

/* Reference constants: chunk.rs:5-17, perlin_util.rs:6-29, world.rs:11-12; seed 0. */
void uww_params_reference(uww_params* p);

/* The seeded 256-entry permutation of noise::Perlin::new(seed) (state.rs:359). */
int uww_perm_table(uint32_t seed, uint8_t out[256]);

/* Fill desc[i].cell_offset / sample_offset with the running sums of cells^3 and
 * (cells+1)^3; the totals go to *total_cells / *total_samples (either may be NULL). */
int uww_layout_cells(uww_chunk_desc* desc, uint32_t n, uint64_t* total_cells, uint64_t* total_samples);

/* ---- context (replaces the noise::Perlin handle passed to every build) ---- */
/* stream: a cudaStream_t, or NULL for a stream the context creates and owns.
 * create and set_params refuse, with UWW_ERR_INVALID_ARG, parameters with a
 * non-finite float, octaves outside 1..UWW_MAX_OCTAVES, chunk_size outside
 * 1..2^20, an unknown mode or output bit, a terraced bias with bias_b or
 * bias_c zero, or an empty colour ramp (color_min_z == color_max_z). */
int   uww_ctx_create(const uww_params* p, void* stream, uww_ctx** out);
int   uww_ctx_destroy(uww_ctx* ctx);
int   uww_ctx_set_params(uww_ctx* ctx, const uww_params* p);
int   uww_ctx_get_params(const uww_ctx* ctx, uww_params* p);
void* uww_ctx_stream(uww_ctx* ctx);
int   uww_ctx_sync(uww_ctx* ctx);

/* ---- chunk builds ------------------------------------------------------------ */
/* Batched build (replaces World's one-chunk-per-frame loop over Chunk::build_partial,
 * world.rs:113-145): every chunk in one call -- a planning kernel, a persistent
 * kernel fed by device work queues and an emission kernel, chained on the
 * context's stream (uww_launch_shape_of names the build a batch takes).
 * d_chunks and out are device memory; max_cells bounds desc.cells and sizes
 * the context's work buffers, which grow to the largest batch (chunks above 16
 * cells: max_cells^2 words of slab seam per slab place); a failed allocation
 * returns UWW_ERR_OOM.  Asynchronous; read out->totals or records after
 * uww_ctx_sync(). */
int uww_build_chunks(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n,
                     uint32_t max_cells, const uww_mesh_out* out);

/* Batched build for callers that cannot allocate device memory.  No
 * counterpart in the reference (its chunks are built on the CPU).  For an
 * engine whose allocator owns all device memory, or code that must not call
 * cudaMalloc on its frame path: no context (creating one allocates) and no
 * allocation of any kind.  The caller passes descriptors and output buffers
 * it already owns; the build's scratch (work-queue counter and the look-back
 * words of the device-wide prefix sum) is a fixed 512 KB array that the
 * library holds on every GPU that loads it, for the life of the process.
 * Limits: n <= 65536 chunks, and each chunk's working set must fit in shared
 * memory (up to about 18 cells per edge); otherwise UWW_ERR_INVALID_ARG.
 * Every call shares that array and clears the part it uses first, so calls
 * that overlap on the GPU race: serialise them.  The first call on a device
 * looks up the array's address and sets kernel attributes; make it before any
 * stream capture.  That set-up is kept for the life of the process, so a
 * cudaDeviceReset() of the device afterwards is not supported.  out->totals
 * is required (UWW_ERR_INVALID_ARG without it): its four words are the only
 * report of a timed-out wait, a bad descriptor or an overflow.  Otherwise as
 * uww_build_chunks, asynchronous on `stream` (a cudaStream_t, NULL for the
 * legacy default stream). */
int uww_build_chunks_noalloc(const uww_params* p, void* stream, const uww_chunk_desc* d_chunks, uint32_t n,
                             uint32_t max_cells, const uww_mesh_out* out);

/* Marching cubes over caller-provided density samples instead of the noise:
 * chunk i reads (cells+1)^3 f32 at d_samples + desc.sample_offset, laid out
 * (x*S + y)*S + z like Build::isos (chunk.rs:43, 351-353).  Otherwise as
 * uww_build_chunks. */
int uww_build_chunks_from_samples(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                                  const float* d_samples, uint64_t sample_count, const uww_mesh_out* out);

/* One chunk per launch: the direct drop-in for Chunk::build_full (chunk.rs:266-268).
 * d_chunk points to one device descriptor whose cells equal `cells`; out
 * describes that chunk's own buffers (offsets in its record are 0) and
 * out->totals is required.  Asynchronous. */
int uww_build_chunk_plain(uww_ctx* ctx, const uww_chunk_desc* d_chunk, uint32_t cells, const uww_mesh_out* out);

/* Host-buffer form of uww_build_chunks: copies the descriptors in, builds,
 * copies records, vertices, normals, indices and cases out, synchronises.
 * With page-locked output buffers (uww_host_alloc, or any memory the device
 * can address) at 4-byte alignment, the build streams each finished chunk to
 * them while later chunks build, and the host synchronises once; other host
 * buffers are filled by sized copies after the build.
 * Returns UWW_ERR_CAPACITY (records still valid) when a capacity is too small. */
int uww_build_chunks_host(uww_ctx* ctx, const uww_chunk_desc* h_chunks, uint32_t n,
                          const uww_mesh_out* h_out);

/* ---- tuning (written by the autotuner; 0 = automatic) ------------------------ */
typedef struct uww_tuning {
    int32_t threads;        /* compute threads per CTA (multiple of 32, <= 192 or 224..512); the
                               pipelined build adds one control warp                        */
    int32_t blocks_per_sm;  /* resident CTAs per SM of the persistent grid                   */
    int32_t smem_cells;     /* chunks up to this many cells per edge work in shared memory;
                               larger ones are built as x slabs (split build) or in a
                               global scratch slot per CTA (pipelined build)                */
    int32_t spin_limit;     /* bound, in SM clock cycles, on each device-side wait of the
                               batched builds (the pipelined build's prefix-sum look-back,
                               the split build's wait for the records); 0 = the default,
                               4e9 cycles (about 2 s).  A wait that runs out raises
                               UWW_ERRFLAG_TIMEOUT and the build finishes without it      */
    uint32_t test_flags;    /* UWW_TEST_*: failure injection for tests; 0 in normal use      */
    uint32_t options;       /* UWW_TUNE_*; 0 in normal use                                   */
    int32_t reserved[2];
} uww_tuning;               /* 32 bytes */

/* uww_tuning.options.  NO_DEPTH_SHORTCUT: evaluate the whole noise of every
 * chunk, also of the chunks whose depth bias alone decides every sample and
 * of those whose first octaves already settle them as blank or solid (the
 * output does not change; for measuring the per-chunk cost of the full
 * path). */
#define UWW_TUNE_NO_DEPTH_SHORTCUT 1u
/* PIPELINED: build every batch with the single pipelined kernel (look-back
 * prefix sum, one CTA emits the chunks it sampled).  By default a batch whose
 * chunks all fit one shared-memory workspace (<= 256 compute threads), or
 * whose chunks above 16 cells per edge (up to 63) can be built as x slabs of
 * a few cell layers, with no streamed host output, no samples read in and no
 * look-back failure injection, takes the split build instead: a planning
 * kernel, the front half of every chunk or slab, then the emission of every
 * vertex and index of the batch.  Both give the same output. */
#define UWW_TUNE_PIPELINED 2u

/* Failure injection (uww_tuning.test_flags).  WITHHOLD_FIRST: the first chunk
 * of every batched build never publishes its prefix, so the look-back waits
 * of the chunks after it run out (after spin_limit cycles each): the build
 * returns with UWW_ERRFLAG_TIMEOUT, every chunk after the first flagged
 * UWW_CHUNK_OVERFLOW and nothing written outside the output capacities.  It
 * lets a test check the timeout path without a fault or a hang. */
#define UWW_TEST_WITHHOLD_FIRST 1u
/* WITHHOLD_RECORDS: in the split build, the records of the batch's first
 * tile of chunks are written but never announced, so every emission unit's
 * wait for the records runs out (after spin_limit cycles): the build returns
 * with UWW_ERRFLAG_TIMEOUT, stores no vertex, normal or index, and writes
 * nothing outside the output capacities.  (The pipelined build, which the
 * look-back flag selects, ignores it.) */
#define UWW_TEST_WITHHOLD_RECORDS 2u
/* The autotuner sets threads, blocks_per_sm and smem_cells and keeps the
 * context's spin_limit and test_flags. */
int uww_ctx_set_tuning(uww_ctx* ctx, const uww_tuning* t);
int uww_ctx_get_tuning(const uww_ctx* ctx, uww_tuning* t);

/* Autotuner (no counterpart in the reference, whose chunk build has no launch
 * shape): times the batched build of these chunks under each candidate tuning
 * -- compute threads per CTA (64..192, and 256..512 when chunks exceed 12
 * cells per edge), CTAs per SM up to the occupancy limit, and the LOD above
 * which chunks work in a global scratch slot instead of shared memory --
 * keeps the fastest, sets it on the context and returns it (*best_us: its
 * time in microseconds).  With cache_path, the result is first looked up in
 * and then appended to that text file, one line per key; the key is the
 * device, the batch size (power of two), the LOD histogram (5 % steps) and
 * the parameters that change the kernel's cost (octaves, outputs, math and
 * dedup modes, normalisation, bias).  Synchronises the context stream; the
 * outputs hold the last timed build.  UWW_ERR_CAPACITY if they overflow. */
int uww_autotune(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                 const uww_mesh_out* out, const char* cache_path, uww_tuning* best, float* best_us);

/* The launch shape a batched build (uww_build_chunks) of n chunks of up to
 * max_cells cells per edge takes with the context's parameters and tuning,
 * for diagnostics and tests (no counterpart in the reference): the build
 * (UWW_BUILD_SPLIT: planning, front and emission kernels; UWW_BUILD_PIPELINED:
 * the single persistent kernel), the most x slabs a chunk is built as (1:
 * every chunk whole; the split build builds chunks of 17 to 63 cells per edge
 * as slabs of a few cell layers), the compute threads
 * per CTA, the (front) kernel's grid, its resident CTAs per SM and its dynamic
 * shared memory.  It assumes per-cell cases and samples are written exactly
 * when the parameters' outputs ask for them. */
#define UWW_BUILD_PIPELINED 0u
#define UWW_BUILD_SPLIT     1u
typedef struct uww_launch_shape {
    uint32_t build;
    uint32_t slabs_per_chunk;
    uint32_t threads;
    uint32_t grid;
    uint32_t blocks_per_sm;
    uint32_t dyn_smem;
} uww_launch_shape;
int uww_launch_shape_of(uww_ctx* ctx, uint32_t n, uint32_t max_cells, uww_launch_shape* out);

/* ---- per-frame build as a CUDA graph -------------------------------------------- */
/* Replaces World::build_step's per-frame slice of chunk builds (world.rs:113-145)
 * with one graph launch: copy h_chunks[0..max_chunks) and *h_count (page-locked
 * host memory the caller fills each frame) to the device, run the batched
 * build over the first *h_count descriptors (the kernel reads the count on
 * the device), and copy the records (if h_records) and totals (if h_totals,
 * page-locked) back.  The mesh stays in d_out's device buffers.  The graph is
 * captured once, on the context stream, with the context's parameters;
 * uww_frame_set_params recaptures it and updates the instantiated graph.
 * The graph reads h_chunks and h_count and writes h_records and h_totals
 * while it runs: fill the next frame's descriptors only after the previous
 * launch has finished (uww_ctx_sync). */
typedef struct uww_frame uww_frame;
int uww_frame_create(uww_ctx* ctx, uint32_t max_chunks, uint32_t max_cells, const uww_chunk_desc* h_chunks,
                     const uint32_t* h_count, const uww_mesh_out* d_out, uww_chunk_record* h_records,
                     uint64_t* h_totals, uww_frame** out);
int uww_frame_launch(uww_frame* f);          /* asynchronous; then uww_ctx_sync */
int uww_frame_set_params(uww_frame* f, const uww_params* p);
int uww_frame_destroy(uww_frame* f);

/* ---- topology-frozen adjoint (no counterpart in the reference) ---------------- */
/* theta = (a_0 .. a_{K-1}, base_freq, offset[0], offset[1], offset[2], iso_level),
 * K = params.octaves, UWW_THETA_COUNT(K) floats.  a_k are the effective
 * per-octave amplitudes (amps[k] with explicit_amps, else amplitude * persistence^k). */
#define UWW_THETA_COUNT(octaves) ((octaves) + 5)

/* Edge id of a vertex: (s << 3) | dir, s = the chunk-local index (x*S + y)*S + z
 * (S = cells + 1) of the sample the vertex is interpolated from (t = 0 there),
 * dir = 0..5 the direction (+x, -x, +y, -y, +z, -z) of the other sample. */
#define UWW_EDGE_SAMPLE(id) ((id) >> 3)
#define UWW_EDGE_DIR(id)    ((id) & 7u)

/* Forward: uww_build_chunks plus d_edge_ids[v] for every output vertex v (indexed
 * like out->verts; out->vert_capacity entries).  With the per-cell cases
 * (UWW_OUT_CASES) this is all the backward keeps: the field is not stored. */
int uww_forward(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                const uww_mesh_out* out, uint32_t* d_edge_ids);

/* Backward of a loss L(vertex positions) with the topology of the forward held
 * fixed.  d_pos_grad = dL/d(position), 3 floats per vertex indexed like the
 * forward's verts; d_records and d_edge_ids are the forward's.  Writes
 * d_theta_grad[UWW_THETA_COUNT(octaves)] = dL/dtheta and, if d_sample_grad is
 * not NULL, dL/d(density sample) at desc.sample_offset (the array is zeroed
 * over sample_capacity floats first).  The density and its analytic spatial
 * and parameter derivatives are recomputed at each vertex's two samples.  The
 * context's parameters must be the forward's.  An edge id outside its chunk
 * makes every theta_grad entry NaN.  Asynchronous. */
int uww_backward(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                 const uww_chunk_record* d_records, const uint32_t* d_edge_ids, const float* d_pos_grad,
                 float* d_theta_grad, float* d_sample_grad, uint64_t sample_capacity);

/* Heightmap loss of the terrain-fitting loop: vertices (count from d_totals[0])
 * are binned into square xy columns of `column` world units starting at
 * (x0, y0), cols_x by cols_y; L = sum over columns holding a vertex of
 * (mean vertex z - d_target[col])^2 / (cols_x * cols_y), col = cy * cols_x + cx.
 * Writes *d_loss and d_pos_grad = dL/d(position) (3 floats per vertex);
 * d_work: 4 * cols_x * cols_y floats of scratch, 8-byte aligned.  The column
 * sums are fixed point (2^-16 world units) with order-independent integer
 * atomics and the loss is reduced in a fixed order, so the result does not
 * change from run to run.  Asynchronous. */
int uww_height_loss(uww_ctx* ctx, const uww_vert_color* d_verts, const uint64_t* d_totals, uint32_t vert_capacity,
                    float x0, float y0, float column, uint32_t cols_x, uint32_t cols_y, const float* d_target,
                    float* d_work, float* d_pos_grad, float* d_loss);

/* ---- memory helpers for callers without their own CUDA binding --------------- */
int uww_device_alloc(size_t bytes, void** out);
int uww_device_free(void* p);
int uww_host_alloc(size_t bytes, void** out);      /* page-locked host memory */
int uww_host_free(void* p);
/* asynchronous on the context stream; kind: 0 host->device, 1 device->host, 2 device->device */
int uww_memcpy(uww_ctx* ctx, void* dst, const void* src, size_t bytes, int kind);
int uww_memset(uww_ctx* ctx, void* dst, int value, size_t bytes);

/* ---- density samples without the mesher -------------------------------------- */
/* Chunk::build_iso (chunk.rs:105-129) for a batch: the (cells+1)^3 f32 density
 * samples of every chunk at d_samples + desc.sample_offset (laid out
 * (x*S + y)*S + z as Build::isos, chunk.rs:351-353), sample_capacity floats
 * available.  The same values as the batched build's UWW_OUT_SAMPLES in the
 * same math mode.  Asynchronous; a descriptor with cells outside 1..max_cells
 * or samples outside the capacity is skipped and flagged (uww_sample_status). */
int uww_sample_chunks(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells, float* d_samples,
                      uint64_t sample_capacity);
/* UWW_ERRFLAG_BAD / UWW_ERRFLAG_RANGE raised by the last uww_sample_chunks (synchronises). */
int uww_sample_status(uww_ctx* ctx, uint32_t* flags);

/* ---- queries against built chunks ---------------------------------------------- */
/* Per-cell triangle ranges for Chunk::tris_around (chunk.rs:315-342): for every
 * cell of every chunk, the chunk-local position in the index buffer of its first
 * triangle (cells are emitted in stream order, 3 * ntri(case) indices each),
 * written at d_first + desc.cell_offset from the build's cases (UWW_OUT_CASES).
 * A chunk whose cells lie outside case_capacity is skipped and flagged
 * (uww_sample_status). */
int uww_cell_tri_offsets(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, const uint8_t* d_cases,
                         uint64_t case_capacity, uint32_t* d_first);

/* Device index of chunk positions (World::get_chunk, world.rs:89-91): an open-
 * addressing table of table_size (a power of two >= n) u32 slots holding
 * chunk index + 1.  A position that appears twice keeps one of its chunks. */
int uww_chunk_index(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t* d_table, uint32_t table_size);

/* A built batch, as the ray query reads it (all device pointers, one build). */
typedef struct uww_ray_scene {
    const uww_chunk_desc*   chunks;
    const uww_chunk_record* records;
    const uww_vert_color*   verts;
    const uint32_t*         inds;
    const uint8_t*          cases;       /* UWW_OUT_CASES of the build                */
    const uint32_t*         cell_first;  /* uww_cell_tri_offsets of those cases        */
    const uint32_t*         table;       /* uww_chunk_index of the chunks              */
    uint32_t                n;
    uint32_t                table_size;
} uww_ray_scene;

/* The boids' wall-avoidance ray casts (boid.rs:175-244), batched: for query q
 * at d_origins[q] (world xyz) and its nrays (<= 32) directions d_dirs[q][k],
 * the triangles of the cells within `range` cells of the point
 * (Chunk::tris_around) in every chunk within `range` world units
 * (boid.rs:176-207) are cast against each ray with util::Tri::intersects
 * (util.rs:23-58, max distance `range`); d_t[q][k] = the nearest hit distance,
 * or -1.  f32 with the reference's operation order (no FMA). */
int uww_ray_query(uww_ctx* ctx, const uww_ray_scene* scene, const float* d_origins, uint32_t nq, const float* d_dirs,
                  uint32_t nrays, int32_t range, float* d_t);

/* ---- the chunk scheduler's feed ------------------------------------------------- */
/* World::update_nearby (world.rs:148-234) on the GPU: every chunk position in
 * the box around the sub (x, y in sub_chunk +- generation_dist, z clamped to
 * [min_z, max_z]) within generation_dist chunk lengths of sub_pos is tested
 * against the two frusta (util::in_frustum, util.rs:77-85: clip = M (p, 1),
 * divide by w, |x|, |y| <= 1, 0 <= z <= 1; M column-major as cgmath's, the
 * camera's chunk_generation_frustum_matrix).  A position with a known chunk
 * (d_known_table: uww_chunk_index of d_known, NULL for none) that has a mesh,
 * lies within view_dist chunk lengths and is in the view frustum goes to
 * d_render (x, y, z triples, loop order); an unknown one goes to d_generate as
 * a descriptor of `cells` cells (offsets laid out as uww_layout_cells), in
 * GenPrio order (world.rs:33-58): in view first, then in the generation
 * frustum, then ascending dist^2 + z, ties by loop order -- the order the
 * batched build's work queue takes, so in-view chunks finish first.
 * d_counts[0], [1]: the lists' true lengths (entries beyond the capacities are
 * not written).  At most 4096 candidate positions. */
typedef struct uww_schedule_params {
    float    sub_pos[3];
    int32_t  sub_chunk[3];
    float    view_proj[16];      /* VIEW_FRUST_FOVY matrix (world.rs:16)      */
    float    gen_proj[16];       /* GENERATE_FRUST_FOVY matrix (world.rs:17)  */
    int32_t  generation_dist;    /* GENERATION_DIST = 5 (world.rs:9)          */
    int32_t  view_dist;          /* VIEW_DIST = 4 (world.rs:8)                */
    int32_t  min_z, max_z;       /* world::MIN_Z, MAX_Z (world.rs:11-12)      */
    uint32_t cells;              /* cells per edge of the generated chunks    */
} uww_schedule_params;
int uww_schedule_chunks(uww_ctx* ctx, const uww_schedule_params* sp, const uww_chunk_desc* d_known,
                        const uww_chunk_record* d_known_records, const uint32_t* d_known_table,
                        uint32_t known_table_size, uww_chunk_desc* d_generate, uint32_t generate_capacity,
                        int32_t* d_render, uint32_t render_capacity, uint32_t* d_counts);

/* ---- terrain shading arithmetic (headless) -------------------------------------- */
/* camera::CameraUniform (camera.rs:69-79): view_proj column-major, fog colour,
 * sub position and forward vector, each vec3 padded to 16 bytes. */
typedef struct uww_camera_uniform {
    float view_proj[16];
    float fog_color[3];
    float pad1;
    float sub_pos[3];
    float pad2;
    float sub_forward[3];
    float pad3;
} uww_camera_uniform;

/* terrain.wgsl (underwater_world/src/terrain.wgsl:26-59) evaluated per vertex
 * into device buffers instead of a render target (no graphics API here):
 * d_clip[v] = view_proj * (pos, 1) (4 floats), d_rgb[v] = fs_main's fogged
 * colour at the vertex (3 floats), d_dist_light[v] = (distance to the sub,
 * smoothstepped spotlight term) (2 floats); any of the three may be NULL.  The
 * vertex count is d_totals[0] (a build's totals, clamped to vert_capacity) or,
 * with d_totals NULL, `count`.  Asynchronous. */
int uww_shade_vertices(uww_ctx* ctx, const uww_camera_uniform* cam, const uww_vert_color* d_verts,
                       const uint64_t* d_totals, uint32_t count, uint32_t vert_capacity, float* d_clip, float* d_rgb,
                       float* d_dist_light);

/* ---- point queries ------------------------------------------------------------ */
/* density(world xyz) for n points: perlin_util::iso_at (perlin_util.rs:24-29) with
 * (x,y,z) = world / CHUNK_SIZE as in boid.rs:132-137.  d_xyz: 3n floats; d_out: n. */
int uww_density_at(uww_ctx* ctx, const float* d_xyz, uint32_t n, float* d_out);

#ifdef __cplusplus
}
#endif
#endif /* UWW_H */
