/*
 * uww_oracle.c -- CPU oracle for the chunk-generation path.
 *
 * TEST INFRASTRUCTURE ONLY.  The CUDA library is verified against this file:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * The product (libuww_gb300.so) never links, calls or falls back to it.
 *
 * It restates, on the CPU, the reference chunk builder of
 * LelsersLasers/UnderwaterWorld:
 *   - noise::Perlin::new(seed) permutation (state.rs:359)   -> oracle_perm
 *   - perlin_util::perlin_3d_octaves / iso_at (perlin_util.rs:6-29) -> density
 *   - Chunk::build_iso (chunk.rs:105-129) sample coordinates and layout
 *     isos[x*169 + y*13 + z] (corner_to_iso_idx, chunk.rs:351-353)
 *   - early_blank_check (chunk.rs:131-133)
 *   - build_mesh (chunk.rs:135-264): case bits, corner order, interpolation,
 *     colour (util.rs:93-153), oriented-pair vertex dedup by linear search
 *     (chunk.rs:233), u16->u32 index stream in cell order x, y, z.
 *
 * Two precisions:
 *   ORACLE_F32  the f32 operation order that the GPU parity build follows
 *               (compiled with -ffp-contract=off: nothing fuses);
 *   ORACLE_F64  the reference's own semantics: f64 noise cast to f32
 *               (perlin_util.rs:26), f32 bias and f32 mesh.
 * and two dedup searches with identical results:
 *   linear      the reference's O(V) position() search per emitted index;
 *   hashed      an open-addressing table (for large LODs in tests).
 *
 * Parity status: the marching-cubes tables are generated from the reference's
 * marching_table.rs and the mesh stage follows chunk.rs line by line; the
 * Perlin core and seeding restate the un-vendored `noise` 0.8.2 crate
 * (rand 0.8 / rand_xorshift 0.3) from their published algorithms.  The
 * reference has no tests or golden vectors, so the noise values are
 * *parity unpinned*: nothing in the reference checks them.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "uww.h"
#include "mc_tables.h"
#include "uww_oracle.h"

/* ---------------------------------------------------------------------------
 * Permutation: noise 0.8.2 PermutationTable::new(seed).
 * The seed bytes form an XorShift128 state (x = 1, y = z = w = seed, little
 * endian), and the identity permutation 0..255 is shuffled by rand 0.8's
 * SliceRandom::shuffle: for i = 255 down to 1, swap(i, uniform(0..=i)), where
 * the bounded draw is the widening-multiply rejection method with
 * zone = (range << clz(range)) - 1.
 * ------------------------------------------------------------------------- */
typedef struct { uint32_t x, y, z, w; } xorshift128;

static uint32_t xs_next(xorshift128* r)
{
    uint32_t t = r->x ^ (r->x << 11);
    r->x = r->y;
    r->y = r->z;
    r->z = r->w;
    r->w = r->w ^ (r->w >> 19) ^ (t ^ (t >> 8));
    return r->w;
}

static uint32_t xs_below(xorshift128* r, uint32_t range)
{
    uint32_t zone = (range << __builtin_clz(range)) - 1u;
    for (;;) {
        uint64_t m = (uint64_t)xs_next(r) * (uint64_t)range;
        if ((uint32_t)m <= zone) return (uint32_t)(m >> 32);
    }
}

void oracle_perm(uint32_t seed, uint8_t P[256])
{
    xorshift128 r = {1u, seed, seed, seed};
    for (int i = 0; i < 256; ++i) P[i] = (uint8_t)i;
    for (uint32_t i = 255; i >= 1; --i) {
        uint32_t j = xs_below(&r, i + 1);
        uint8_t t = P[i];
        P[i] = P[j];
        P[j] = t;
    }
}

/* --------------------------------------------------------------------------- */
#define REAL float
#define SUFFIX _f32
#define FLOOR floorf
#include "oracle_noise.inc"
#undef REAL
#undef SUFFIX
#undef FLOOR

#define REAL double
#define SUFFIX _f64
#define FLOOR floor
#include "oracle_noise.inc"
#undef REAL
#undef SUFFIX
#undef FLOOR

/* chunk.rs:14-17 */
#define MIN_HUE (-150.0f)
#define MAX_HUE 60.0f
#define SATURATION 0.6f
#define BASE_VALUE 0.4f

typedef struct {
    const uww_params* p;
    uint8_t P[256];
    float mult32[UWW_MAX_OCTAVES], amp32[UWW_MAX_OCTAVES];
    double mult64[UWW_MAX_OCTAVES], amp64[UWW_MAX_OCTAVES];
} oracle_world;

static void world_init(oracle_world* w, const uww_params* p)
{
    w->p = p;
    oracle_perm(p->seed, w->P);
    octave_tables_f32(p, w->mult32, w->amp32);
    octave_tables_f64(p, w->mult64, w->amp64);
}

/* iso_at (perlin_util.rs:24-29) generalised by bias_mode.  World position is
 * given twice: as the f32 the GPU sees and as the f64 the reference sees. */
static float density_f32(const oracle_world* w, float wx, float wy, float wz, float* grad)
{
    const uww_params* p = w->p;
    float nx = (wx + p->offset[0]) * p->base_freq;
    float ny = (wy + p->offset[1]) * p->base_freq;
    float nz = (wz + p->offset[2]) * p->base_freq;
    float g[3];
    float f = fbm_f32(w->P, p, w->mult32, w->amp32, nx, ny, nz, grad ? g : NULL);
    if (grad) {
        grad[0] = g[0] * p->base_freq;
        grad[1] = g[1] * p->base_freq;
        grad[2] = g[2] * p->base_freq;
    }
    if (p->bias_mode == UWW_BIAS_TERRACED) {
        float adj = nz * p->bias_a / p->bias_b;
        return adj + f - fmodf(adj, p->bias_c);
    }
    if (p->bias_mode == UWW_BIAS_LINEAR) {
        if (grad) grad[2] = grad[2] + p->bias_a;
        return f + p->bias_a * (wz - p->bias_b);
    }
    return f;
}

static float density_f64(const oracle_world* w, double wx, double wy, double wz, float* grad)
{
    const uww_params* p = w->p;
    double nx = (wx + (double)p->offset[0]) * (double)p->base_freq;
    double ny = (wy + (double)p->offset[1]) * (double)p->base_freq;
    double nz = (wz + (double)p->offset[2]) * (double)p->base_freq;
    double g[3];
    float f = (float)fbm_f64(w->P, p, w->mult64, w->amp64, nx, ny, nz, grad ? g : NULL);
    if (grad) {
        grad[0] = (float)(g[0] * (double)p->base_freq);
        grad[1] = (float)(g[1] * (double)p->base_freq);
        grad[2] = (float)(g[2] * (double)p->base_freq);
    }
    if (p->bias_mode == UWW_BIAS_TERRACED) {
        float adj = (float)nz * p->bias_a / p->bias_b;
        return adj + f - fmodf(adj, p->bias_c);
    }
    if (p->bias_mode == UWW_BIAS_LINEAR) {
        if (grad) grad[2] = grad[2] + p->bias_a;
        return f + p->bias_a * ((float)wz - p->bias_b);
    }
    return f;
}

/* Full-f64 density (no f32 cast anywhere) for gradient checks. */
double oracle_density64_full(const uww_params* p, const uint8_t* P, double wx, double wy, double wz,
                             double* grad)
{
    double mult[UWW_MAX_OCTAVES], amp[UWW_MAX_OCTAVES];
    octave_tables_f64(p, mult, amp);
    double nx = (wx + (double)p->offset[0]) * (double)p->base_freq;
    double ny = (wy + (double)p->offset[1]) * (double)p->base_freq;
    double nz = (wz + (double)p->offset[2]) * (double)p->base_freq;
    double g[3];
    double f = fbm_f64(P, p, mult, amp, nx, ny, nz, grad ? g : NULL);
    if (grad) {
        grad[0] = g[0] * (double)p->base_freq;
        grad[1] = g[1] * (double)p->base_freq;
        grad[2] = g[2] * (double)p->base_freq;
    }
    if (p->bias_mode == UWW_BIAS_TERRACED) {
        double adj = nz * (double)p->bias_a / (double)p->bias_b;
        return adj + f - fmod(adj, (double)p->bias_c);
    }
    if (p->bias_mode == UWW_BIAS_LINEAR) {
        if (grad) grad[2] += (double)p->bias_a;
        return f + (double)p->bias_a * (wz - (double)p->bias_b);
    }
    return f;
}

/* --------------------------------------------------------------------------- */
/* util.rs:93-95 */
static float create_mix_ratio(float mn, float mx, float x) { return (x - mn) / (mx - mn); }

/* util.rs:106-112 */
static void to_srgb(const float c[3], float out[3])
{
    for (int i = 0; i < 3; ++i) out[i] = powf((c[i] / 255.0f + 0.055f) / 1.055f, 2.4f);
}

/* util.rs:122-153 */
static void hsv_to_rgb(float hue, float saturation, float value, float out[3])
{
    float r0 = fmodf(hue, 360.0f);
    hue = r0 < 0.0f ? r0 + 360.0f : r0; /* f32::rem_euclid */
    float c = value * saturation;
    float h = hue / 60.0f;
    float x = c * (1.0f - fabsf(fmodf(h, 2.0f) - 1.0f));
    float m = value - c;
    float r, g, b;
    if (0.0f <= h && h < 1.0f)      { r = c; g = x; b = 0.0f; }
    else if (1.0f <= h && h < 2.0f) { r = x; g = c; b = 0.0f; }
    else if (2.0f <= h && h < 3.0f) { r = 0.0f; g = c; b = x; }
    else if (3.0f <= h && h < 4.0f) { r = 0.0f; g = x; b = c; }
    else if (4.0f <= h && h < 5.0f) { r = x; g = 0.0f; b = c; }
    else                            { r = c; g = 0.0f; b = x; }
    out[0] = (r + m) * 255.0f;
    out[1] = (g + m) * 255.0f;
    out[2] = (b + m) * 255.0f;
}

/* --------------------------------------------------------------------------- */
/* Growable per-chunk buffers, like the reference's Vecs (chunk.rs:33-45). */
typedef struct {
    float* verts;      /* 6 floats per vertex: pos, colour */
    float* normals;    /* 3 floats per vertex              */
    uint32_t* inds;
    uint64_t* keys;    /* vert_pairs: (corner a, corner b) packed */
    uint32_t nv, ni, capv, capi;
    uint32_t flags, active;
    /* hashed dedup table */
    uint64_t* hkeys;
    uint32_t* hvals;
    uint32_t hcap;
} chunk_build;

static void cb_reserve(chunk_build* b, uint32_t nv, uint32_t ni)
{
    if (nv > b->capv) {
        uint32_t c = b->capv ? b->capv : 64;
        while (c < nv) c *= 2;
        b->verts = (float*)realloc(b->verts, (size_t)c * 6 * sizeof(float));
        b->normals = (float*)realloc(b->normals, (size_t)c * 3 * sizeof(float));
        b->keys = (uint64_t*)realloc(b->keys, (size_t)c * sizeof(uint64_t));
        b->capv = c;
    }
    if (ni > b->capi) {
        uint32_t c = b->capi ? b->capi : 256;
        while (c < ni) c *= 2;
        b->inds = (uint32_t*)realloc(b->inds, (size_t)c * sizeof(uint32_t));
        b->capi = c;
    }
}

static void cb_free(chunk_build* b)
{
    free(b->verts); free(b->normals); free(b->inds); free(b->keys);
    free(b->hkeys); free(b->hvals);
    memset(b, 0, sizeof(*b));
}

static uint64_t mix64(uint64_t k)
{
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
    return k;
}

/* returns existing id or UINT32_MAX (and inserts nv as the new id) */
static uint32_t hash_find_insert(chunk_build* b, uint64_t key, uint32_t new_id)
{
    if (2u * (b->nv + 1u) > b->hcap) {
        uint32_t nc = b->hcap ? b->hcap * 2 : 1024;
        uint64_t* nk = (uint64_t*)malloc((size_t)nc * sizeof(uint64_t));
        uint32_t* nvv = (uint32_t*)malloc((size_t)nc * sizeof(uint32_t));
        for (uint32_t i = 0; i < nc; ++i) nk[i] = UINT64_MAX;
        for (uint32_t i = 0; i < b->hcap; ++i) {
            if (b->hkeys[i] == UINT64_MAX) continue;
            uint32_t s = (uint32_t)mix64(b->hkeys[i]) & (nc - 1);
            while (nk[s] != UINT64_MAX) s = (s + 1) & (nc - 1);
            nk[s] = b->hkeys[i];
            nvv[s] = b->hvals[i];
        }
        free(b->hkeys); free(b->hvals);
        b->hkeys = nk; b->hvals = nvv; b->hcap = nc;
    }
    uint32_t s = (uint32_t)mix64(key) & (b->hcap - 1);
    while (b->hkeys[s] != UINT64_MAX) {
        if (b->hkeys[s] == key) return b->hvals[s];
        s = (s + 1) & (b->hcap - 1);
    }
    b->hkeys[s] = key;
    b->hvals[s] = new_id;
    return UINT32_MAX;
}

/* chunk.rs:144-153 corner offsets */
static const int CORNER[8][3] = {
    {0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1},
    {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};

typedef struct {
    const oracle_world* w;
    int precision;      /* ORACLE_F32 / ORACLE_F64 */
    int search;         /* ORACLE_SEARCH_LINEAR / ORACLE_SEARCH_HASHED */
} build_cfg;

/* Build one chunk: build_iso + early_blank_check + build_mesh. */
static void build_chunk(const build_cfg* cfg, const uww_chunk_desc* d, chunk_build* b, uint8_t* cases,
                        float* isos_out, const float* isos_in)
{
    const uww_params* p = cfg->w->p;
    const int N = (int)d->cells, S = N + 1;
    const float s = (float)p->chunk_size / (float)N; /* SIZE_SCALE (chunk.rs:7) */
    const int ox = d->pos[0] * p->chunk_size, oy = d->pos[1] * p->chunk_size, oz = d->pos[2] * p->chunk_size;
    const float iso_level = p->iso_level;
    float* isos = isos_out ? isos_out : (float*)malloc((size_t)S * S * S * sizeof(float));

    /* build_iso (chunk.rs:105-129): isos[x*S*S + y*S + z] */
    int any_inside = 0;
    for (int x = 0; x < S; ++x)
        for (int y = 0; y < S; ++y)
            for (int z = 0; z < S; ++z) {
                float v;
                if (isos_in) {
                    v = isos_in[(x * S + y) * S + z];
                } else if (cfg->precision == ORACLE_F32) {
                    float wx = (float)x * s + (float)ox;
                    float wy = (float)y * s + (float)oy;
                    float wz = (float)z * s + (float)oz;
                    v = density_f32(cfg->w, wx, wy, wz, NULL);
                } else {
                    double wx = (double)x * (double)s + (double)ox;
                    double wy = (double)y * (double)s + (double)oy;
                    double wz = (double)z * (double)s + (double)oz;
                    v = density_f64(cfg->w, wx, wy, wz, NULL);
                }
                isos[(x * S + y) * S + z] = v;
                if (!(v > iso_level)) any_inside = 1;
            }

    b->nv = b->ni = 0;
    b->flags = 0;
    b->active = 0;
    if (b->hkeys) for (uint32_t i = 0; i < b->hcap; ++i) b->hkeys[i] = UINT64_MAX;

    if (!any_inside) { /* early_blank_check: every iso > ISO_LEVEL */
        b->flags = UWW_CHUNK_EARLY_BLANK;
        if (cases) memset(cases, 0, (size_t)N * N * N);
        if (!isos_out) free(isos);
        return;
    }

    const int want_color = (p->outputs & UWW_OUT_COLOR) != 0;
    const int want_normals = (p->outputs & UWW_OUT_NORMALS) != 0;
    const uint64_t S3 = (uint64_t)S * S * S;

    /* build_mesh (chunk.rs:135-264), cells x outer, y, z inner */
    for (int x = 0; x < N; ++x)
        for (int y = 0; y < N; ++y)
            for (int z = 0; z < N; ++z) {
                int cc[8][3];
                int tri_idx = 0;
                for (int i = 0; i < 8; ++i) {
                    cc[i][0] = x + CORNER[i][0];
                    cc[i][1] = y + CORNER[i][1];
                    cc[i][2] = z + CORNER[i][2];
                    if (isos[(cc[i][0] * S + cc[i][1]) * S + cc[i][2]] < iso_level) tri_idx |= 1 << i;
                }
                if (cases) cases[(x * N + y) * N + z] = (uint8_t)tri_idx;
                const int8_t* row = UWW_TRI_TABLE[tri_idx];
                if (row[0] >= 0) b->active++;
                for (int i = 0; i < 16 && row[i] >= 0; ++i) {
                    int ca = UWW_EDGE_CORNERS[row[i]][0], cb = UWW_EDGE_CORNERS[row[i]][1];
                    const int* A = cc[ca];
                    const int* B = cc[cb];
                    uint64_t la = ((uint64_t)A[0] * S + A[1]) * S + A[2];
                    uint64_t lb = ((uint64_t)B[0] * S + B[1]) * S + B[2];
                    uint64_t key;
                    if (p->dedup_mode == UWW_DEDUP_EDGE) key = la < lb ? la * S3 + lb : lb * S3 + la;
                    else key = la * S3 + lb;

                    uint32_t ind = UINT32_MAX;
                    if (cfg->search == ORACLE_SEARCH_LINEAR) {
                        /* vert_pairs.iter().position(..) (chunk.rs:233) */
                        for (uint32_t k = 0; k < b->nv; ++k)
                            if (b->keys[k] == key) { ind = k; break; }
                    } else {
                        ind = hash_find_insert(b, key, b->nv);
                    }
                    if (ind == UINT32_MAX) {
                        ind = b->nv;
                        cb_reserve(b, b->nv + 1, 0);
                        float sa[3] = {(float)A[0] * s, (float)A[1] * s, (float)A[2] * s};
                        float sb[3] = {(float)B[0] * s, (float)B[1] * s, (float)B[2] * s};
                        float ia = isos[la], ib = isos[lb];
                        float t = (iso_level - ia) / (ib - ia);
                        float diff[3] = {sb[0] - sa[0], sb[1] - sa[1], sb[2] - sa[2]};
                        float mid[3] = {sa[0] + t * diff[0], sa[1] + t * diff[1], sa[2] + t * diff[2]};
                        float world_z = mid[2] + (float)oz;
                        float* v = b->verts + (size_t)ind * 6;
                        v[0] = mid[0] + (float)ox;
                        v[1] = mid[1] + (float)oy;
                        v[2] = world_z;
                        if (want_color) {
                            float ratio = world_z / (float)p->chunk_size;
                            float mix = create_mix_ratio(p->color_min_z, p->color_max_z, ratio);
                            float vi = (float)(cb % 3) / 9.0f;
                            float hue = MIN_HUE + (MAX_HUE - MIN_HUE) * mix;
                            float rgb[3];
                            hsv_to_rgb(hue, SATURATION, BASE_VALUE + vi, rgb);
                            to_srgb(rgb, v + 3);
                        } else {
                            v[3] = v[4] = v[5] = 0.0f;
                        }
                        float* nrm = b->normals + (size_t)ind * 3;
                        if (want_normals) {
                            float g[3];
                            if (cfg->precision == ORACLE_F32) density_f32(cfg->w, v[0], v[1], v[2], g);
                            else density_f64(cfg->w, (double)v[0], (double)v[1], (double)v[2], g);
                            float mag = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
                            if (mag == 0.0f) { nrm[0] = g[0]; nrm[1] = g[1]; nrm[2] = g[2]; }
                            else { nrm[0] = g[0] / mag; nrm[1] = g[1] / mag; nrm[2] = g[2] / mag; }
                        } else {
                            nrm[0] = nrm[1] = nrm[2] = 0.0f;
                        }
                        b->keys[ind] = key;
                        b->nv++;
                    }
                    cb_reserve(b, 0, b->ni + 1);
                    b->inds[b->ni++] = ind;
                }
            }
    if (b->ni > 0) b->flags |= UWW_CHUNK_HAS_MESH;
    if (!isos_out) free(isos);
}

/* --------------------------------------------------------------------------- */
typedef struct {
    const build_cfg* cfg;
    const uww_chunk_desc* chunks;
    uint32_t n;
    chunk_build* builds;
    uint8_t** cases_at;
    float** samples_out_at;
    const float** samples_in_at;
    volatile uint32_t* next;
    pthread_mutex_t* mu;
} worker_args;

static void* worker(void* arg)
{
    worker_args* a = (worker_args*)arg;
    for (;;) {
        pthread_mutex_lock(a->mu);
        uint32_t i = *a->next;
        *a->next = i + 1;
        pthread_mutex_unlock(a->mu);
        if (i >= a->n) break;
        build_chunk(a->cfg, &a->chunks[i], &a->builds[i], a->cases_at[i], a->samples_out_at[i], a->samples_in_at[i]);
    }
    return NULL;
}

int oracle_build_chunks(const uww_params* p, int precision, int search, const uww_chunk_desc* chunks,
                        uint32_t n, const uww_mesh_out* out, int threads, const float* samples_in,
                        uint64_t samples_in_count)
{
    if (!p || (!chunks && n) || !out || !out->records) return UWW_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; ++i)
        if (chunks[i].cells < 1 || chunks[i].cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    oracle_world w;
    world_init(&w, p);
    build_cfg cfg = {&w, precision, search};
    chunk_build* builds = (chunk_build*)calloc(n ? n : 1, sizeof(chunk_build));
    if (!builds) return UWW_ERR_OOM;
    uint8_t* cases = (p->outputs & UWW_OUT_CASES) ? out->cases : NULL;
    float* samples_out = (p->outputs & UWW_OUT_SAMPLES) ? out->samples : NULL;
    /* per-chunk pointers, each checked against the capacity it writes into */
    uint8_t** cases_at = (uint8_t**)calloc(n ? n : 1, sizeof(uint8_t*));
    float** so_at = (float**)calloc(n ? n : 1, sizeof(float*));
    const float** si_at = (const float**)calloc(n ? n : 1, sizeof(float*));
    uint64_t errflags = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint64_t c = chunks[i].cells, nc = c * c * c, ns = (c + 1) * (c + 1) * (c + 1);
        if (samples_in) {
            if (chunks[i].sample_offset + ns > samples_in_count) { free(builds); free(cases_at); free(so_at); free(si_at); return UWW_ERR_INVALID_ARG; }
            si_at[i] = samples_in + chunks[i].sample_offset;
        }
        if (cases) {
            if (chunks[i].cell_offset + nc <= out->case_capacity) cases_at[i] = cases + chunks[i].cell_offset;
            else errflags |= UWW_ERRFLAG_RANGE;
        }
        if (samples_out) {
            if (chunks[i].sample_offset + ns <= out->sample_capacity) so_at[i] = samples_out + chunks[i].sample_offset;
            else errflags |= UWW_ERRFLAG_RANGE;
        }
    }

    if (threads <= 1 || n <= 1) {
        for (uint32_t i = 0; i < n; ++i) build_chunk(&cfg, &chunks[i], &builds[i], cases_at[i], so_at[i], si_at[i]);
    } else {
        volatile uint32_t next = 0;
        pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
        worker_args a = {&cfg, chunks, n, builds, cases_at, so_at, si_at, &next, &mu};
        pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
        for (int t = 0; t < threads; ++t) pthread_create(&tid[t], NULL, worker, &a);
        for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
        free(tid);
    }

    /* compact, in chunk order, exactly as the GPU lays the batch out */
    uint64_t vo = 0, io = 0, overflow = 0;
    int status = UWW_OK;
    for (uint32_t i = 0; i < n; ++i) {
        chunk_build* b = &builds[i];
        uww_chunk_record* r = &out->records[i];
        memset(r, 0, sizeof(*r));
        r->num_verts = b->nv;
        r->num_inds = b->ni;
        r->vert_offset = (uint32_t)vo;
        r->ind_offset = (uint32_t)io;
        r->flags = b->flags;
        r->num_active_cells = b->active;
        if (vo + b->nv > out->vert_capacity || io + b->ni > out->ind_capacity) {
            r->flags |= UWW_CHUNK_OVERFLOW;
            overflow++;
            status = UWW_ERR_CAPACITY;
        } else {
            if (out->verts && b->nv) memcpy(out->verts + vo, b->verts, (size_t)b->nv * 6 * sizeof(float));
            if (out->normals && b->nv) memcpy(out->normals + vo * 3, b->normals, (size_t)b->nv * 3 * sizeof(float));
            if (out->inds && b->ni) memcpy(out->inds + io, b->inds, (size_t)b->ni * sizeof(uint32_t));
        }
        vo += b->nv;
        io += b->ni;
        cb_free(b);
    }
    if (out->totals) {
        out->totals[0] = vo;
        out->totals[1] = io;
        out->totals[2] = overflow;
        out->totals[3] = errflags;
    }
    free(builds);
    free(cases_at);
    free(so_at);
    free(si_at);
    if (errflags && status == UWW_OK) status = UWW_ERR_INVALID_ARG;
    return status;
}

int oracle_sample_grid(const uww_params* p, int precision, const uww_chunk_desc* d, float* isos)
{
    if (!p || !d || !isos || d->cells < 1 || d->cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    oracle_world w;
    world_init(&w, p);
    build_cfg cfg = {&w, precision, ORACLE_SEARCH_HASHED};
    chunk_build b;
    memset(&b, 0, sizeof(b));
    /* sampling only: run with an iso-level above everything so no mesh is built */
    uww_params q = *p;
    q.iso_level = -INFINITY;
    w.p = &q;
    build_chunk(&cfg, d, &b, NULL, isos, NULL);
    cb_free(&b);
    return UWW_OK;
}

int oracle_density_at(const uww_params* p, int precision, const float* xyz, uint32_t n, float* out,
                      float* grad)
{
    if (!p || (n && (!xyz || !out))) return UWW_ERR_INVALID_ARG;
    oracle_world w;
    world_init(&w, p);
    for (uint32_t i = 0; i < n; ++i) {
        float* g = grad ? grad + 3 * (size_t)i : NULL;
        if (precision == ORACLE_F32) out[i] = density_f32(&w, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], g);
        else out[i] = density_f64(&w, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], g);
    }
    return UWW_OK;
}

int oracle_perlin(uint32_t seed, int precision, const double* xyz, uint32_t n, double* out)
{
    uint8_t P[256];
    oracle_perm(seed, P);
    for (uint32_t i = 0; i < n; ++i) {
        if (precision == ORACLE_F32)
            out[i] = (double)perlin_f32(P, (float)xyz[3 * i], (float)xyz[3 * i + 1], (float)xyz[3 * i + 2], NULL);
        else
            out[i] = perlin_f64(P, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], NULL);
    }
    return UWW_OK;
}
