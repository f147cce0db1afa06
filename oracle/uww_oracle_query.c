/*
 * uww_oracle_query.c -- CPU restatement of the queries against built chunks
 * (uww_cell_tri_offsets / uww_ray_query of libuww_gb300.so).
 * TEST INFRASTRUCTURE ONLY: the product never links this file.
 *
 * Follows, in f32 with every operation separately rounded (the Makefile
 * builds with -ffp-contract=off; Rust's cgmath does not fuse either):
 *   boid.rs:175-207   the chunk window around a boid and the local position
 *                     handed to tris_around;
 *   chunk.rs:315-342  Chunk::tris_around, the cells within `range` of it;
 *   util.rs:12-21     Tri::new, face normal safe_normalize((b-a) x (c-a));
 *   util.rs:23-58     Tri::intersects, the hit distance along a ray.
 * A cell's triangles are the build's indices 3*ntri(case) at the cell's
 * running offset in stream order (the order build_mesh visits cells,
 * chunk.rs:135-264).  The nearest hit per ray is what boid.rs:209-244 needs:
 * it tests "some hit closer than the range" and "no hit within the range".
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "uww.h"
#include "mc_tables.h"
#include "uww_oracle.h"

typedef struct {
    float x, y, z;
} v3;

static v3 sub3(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static float dot3(v3 a, v3 b)
{
    float r = a.x * b.x;
    r = r + a.y * b.y;
    return r + a.z * b.z;
}
static v3 cross3(v3 a, v3 b)
{
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}

/* util.rs:23-58 */
static float tri_intersects(v3 a, v3 b, v3 c, v3 n, v3 o, v3 d, float range)
{
    const float dn = dot3(n, d);
    if (fabsf(dn) < 1e-5f) return -1.f;
    const float t = dot3(n, sub3(a, o)) / dn;
    if (t < 0.f || t > range) return -1.f;
    v3 p = {o.x + d.x * t, o.y + d.y * t, o.z + d.z * t};
    const float d0 = dot3(cross3(sub3(b, a), sub3(p, a)), n);
    const float d1 = dot3(cross3(sub3(c, b), sub3(p, b)), n);
    const float d2 = dot3(cross3(sub3(a, c), sub3(p, c)), n);
    if (d0 >= 0.f && d1 >= 0.f && d2 >= 0.f) return t == 0.f ? 0.f : t;
    return -1.f;
}

int oracle_cell_tri_offsets(const uww_chunk_desc* chunks, uint32_t n, const uint8_t* cases, uint32_t* first)
{
    for (uint32_t c = 0; c < n; ++c) {
        const uint64_t NC = (uint64_t)chunks[c].cells * chunks[c].cells * chunks[c].cells;
        uint32_t run = 0;
        for (uint64_t i = 0; i < NC; ++i) {
            first[chunks[c].cell_offset + i] = run;
            run += 3u * UWW_CASE_NTRI[cases[chunks[c].cell_offset + i]];
        }
    }
    return UWW_OK;
}

int oracle_ray_query(const uww_params* p, const uww_chunk_desc* chunks, uint32_t n, const uww_chunk_record* records,
                     const uww_vert_color* verts, const uint32_t* inds, const uint8_t* cases, const float* origins,
                     uint32_t nq, const float* dirs, uint32_t nrays, int32_t range, float* out)
{
    const float cs = (float)p->chunk_size, rf = (float)range;
    uint32_t* first = NULL;
    uint64_t total = 0;
    for (uint32_t c = 0; c < n; ++c) {
        const uint64_t e = chunks[c].cell_offset + (uint64_t)chunks[c].cells * chunks[c].cells * chunks[c].cells;
        if (e > total) total = e;
    }
    first = (uint32_t*)malloc((size_t)(total ? total : 1) * sizeof(uint32_t));
    if (!first) return UWW_ERR_OOM;
    oracle_cell_tri_offsets(chunks, n, cases, first);
    for (uint32_t q = 0; q < nq; ++q) {
        const v3 o = {origins[3 * q], origins[3 * q + 1], origins[3 * q + 2]};
        for (uint32_t k = 0; k < nrays; ++k) out[(size_t)q * nrays + k] = -1.f;
        /* boid.rs:176-182 */
        const int sx = (int)floorf((o.x - rf) / cs), ex = (int)floorf((o.x + rf) / cs);
        const int sy = (int)floorf((o.y - rf) / cs), ey = (int)floorf((o.y + rf) / cs);
        const int sz = (int)floorf((o.z - rf) / cs), ez = (int)floorf((o.z + rf) / cs);
        for (int a = sx; a <= ex; ++a)
            for (int b = sy; b <= ey; ++b)
                for (int cz = sz; cz <= ez; ++cz) {
                    int ci = -1; /* World::get_chunk */
                    for (uint32_t i = 0; i < n; ++i)
                        if (chunks[i].pos[0] == a && chunks[i].pos[1] == b && chunks[i].pos[2] == cz) { ci = (int)i; break; }
                    if (ci < 0) continue;
                    const uww_chunk_desc* d = &chunks[ci];
                    const uww_chunk_record* r = &records[ci];
                    if (!(r->flags & UWW_CHUNK_HAS_MESH) || (r->flags & UWW_CHUNK_OVERFLOW)) continue;
                    const int N = (int)d->cells;
                    const float nf = (float)N;
                    /* boid.rs:185-204: local position as a fraction of the chunk */
                    const float px = (o.x - (float)a * cs) / cs;
                    const float py = (o.y - (float)b * cs) / cs;
                    const float pz = (o.z - (float)cz * cs) / cs;
                    /* chunk.rs:316-326 */
                    const int mx = (int)floorf(px * nf), my = (int)floorf(py * nf), mz = (int)floorf(pz * nf);
                    const int x0 = mx - range > 0 ? mx - range : 0, y0 = my - range > 0 ? my - range : 0,
                              z0 = mz - range > 0 ? mz - range : 0;
                    const int x1 = mx + range < N - 1 ? mx + range : N - 1, y1 = my + range < N - 1 ? my + range : N - 1,
                              z1 = mz + range < N - 1 ? mz + range : N - 1;
                    for (int x = x0; x <= x1; ++x)
                        for (int y = y0; y <= y1; ++y)
                            for (int z = z0; z <= z1; ++z) {
                                const uint32_t cell = d->cell_offset + (uint32_t)((x * N + y) * N + z);
                                const int nt = UWW_CASE_NTRI[cases[cell]];
                                const uint32_t f = r->ind_offset + first[cell];
                                for (int j = 0; j < nt; ++j) {
                                    v3 vv[3];
                                    for (int m = 0; m < 3; ++m) {
                                        const uww_vert_color* vc = &verts[r->vert_offset + inds[f + 3 * j + m]];
                                        vv[m].x = vc->pos[0];
                                        vv[m].y = vc->pos[1];
                                        vv[m].z = vc->pos[2];
                                    }
                                    /* util.rs:12-21 */
                                    v3 nn = cross3(sub3(vv[1], vv[0]), sub3(vv[2], vv[0]));
                                    const float mag = sqrtf(dot3(nn, nn));
                                    if (mag != 0.f) { nn.x = nn.x / mag; nn.y = nn.y / mag; nn.z = nn.z / mag; }
                                    for (uint32_t k = 0; k < nrays; ++k) {
                                        const size_t di = 3 * ((size_t)q * nrays + k);
                                        const v3 dir = {dirs[di], dirs[di + 1], dirs[di + 2]};
                                        const float t = tri_intersects(vv[0], vv[1], vv[2], nn, o, dir, rf);
                                        float* best = &out[(size_t)q * nrays + k];
                                        if (t >= 0.f && (*best < 0.f || t < *best)) *best = t;
                                    }
                                }
                            }
                }
    }
    free(first);
    return UWW_OK;
}

/* ---- World::update_nearby (world.rs:148-234) ---------------------------------- */
static int in_frustum_f(const float* m, float x, float y, float z)
{
    float c[4];
    for (int i = 0; i < 4; ++i) {
        float r = m[i] * x;
        r = r + m[4 + i] * y;
        r = r + m[8 + i] * z;
        c[i] = r + m[12 + i] * 1.0f;
    }
    const float w = c[3];
    const float cx = c[0] / w, cy = c[1] / w, cz = c[2] / w;
    return fabsf(cx) <= 1.0f && fabsf(cy) <= 1.0f && cz >= 0.0f && cz <= 1.0f;
}

typedef struct {
    int cls;
    float prio;
    int idx;
} gen_entry;

static int gen_cmp(const void* a, const void* b)
{
    const gen_entry* x = (const gen_entry*)a;
    const gen_entry* y = (const gen_entry*)b;
    if (x->cls != y->cls) return x->cls < y->cls ? -1 : 1;
    if (x->prio != y->prio) return x->prio < y->prio ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

int oracle_schedule_chunks(const uww_params* p, const uww_schedule_params* sp, const uww_chunk_desc* known,
                           const uww_chunk_record* known_records, uint32_t n_known, uww_chunk_desc* gen_out,
                           uint32_t gen_cap, int32_t* render_out, uint32_t render_cap, uint32_t* counts)
{
    const int G = sp->generation_dist;
    const int sz = sp->sub_chunk[2] - G > sp->min_z ? sp->sub_chunk[2] - G : sp->min_z;
    const int ez = sp->sub_chunk[2] + G < sp->max_z ? sp->sub_chunk[2] + G : sp->max_z;
    const int nz = ez - sz + 1 > 0 ? ez - sz + 1 : 0;
    const float cs = (float)p->chunk_size;
    const float max_view = (float)sp->view_dist * cs, max_gen = (float)G * cs;
    const int total = 4 * G * G * nz;
    gen_entry* gens = (gen_entry*)malloc((size_t)(total ? total : 1) * sizeof(gen_entry));
    if (!gens) return UWW_ERR_OOM;
    uint32_t ng = 0, nr = 0;
    int i = 0;
    for (int x = -G; x < G; ++x)
        for (int y = -G; y < G; ++y)
            for (int z = sz; z <= ez; ++z, ++i) {
                const int cx = sp->sub_chunk[0] + x, cy = sp->sub_chunk[1] + y;
                const float mx = ((float)cx + 0.5f) * cs, my = ((float)cy + 0.5f) * cs, mz = ((float)z + 0.5f) * cs;
                const float dx = sp->sub_pos[0] - mx, dy = sp->sub_pos[1] - my, dz = sp->sub_pos[2] - mz;
                float d2 = dx * dx;
                d2 = d2 + dy * dy;
                d2 = d2 + dz * dz;
                const float dist = sqrtf(d2);
                if (dist > max_gen) continue;
                int in_view = 0, in_gen = 0;
                static const float corners[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                                    {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
                for (int k = 0; k < 8; ++k) {
                    const float px = ((float)cx + corners[k][0]) * cs, py = ((float)cy + corners[k][1]) * cs,
                                pz = ((float)z + corners[k][2]) * cs;
                    if (in_frustum_f(sp->gen_proj, px, py, pz)) {
                        in_gen = 1;
                        if (in_frustum_f(sp->view_proj, px, py, pz)) { in_view = 1; break; }
                    }
                }
                int kc = -1; /* World::get_chunk */
                for (uint32_t j = 0; j < n_known; ++j)
                    if (known[j].pos[0] == cx && known[j].pos[1] == cy && known[j].pos[2] == z) { kc = (int)j; break; }
                if (kc >= 0) {
                    const int not_blank = (known_records[kc].flags & UWW_CHUNK_HAS_MESH) != 0;
                    if (dist < max_view && not_blank && in_view) {
                        if (nr < render_cap) {
                            render_out[3 * nr] = cx;
                            render_out[3 * nr + 1] = cy;
                            render_out[3 * nr + 2] = z;
                        }
                        ++nr;
                    }
                } else {
                    gens[ng].cls = in_view ? 0 : in_gen ? 1 : 2;
                    gens[ng].prio = dist * dist + (float)z * cs;
                    gens[ng].idx = i;
                    ++ng;
                }
            }
    /* GenPrio order: the reference sorts descending and pops from the end */
    qsort(gens, ng, sizeof(gen_entry), gen_cmp);
    const uint32_t cells = sp->cells, nc = cells * cells * cells, ns = (cells + 1) * (cells + 1) * (cells + 1);
    for (uint32_t r = 0; r < ng && r < gen_cap; ++r) {
        const int idx = gens[r].idx;
        const int xi = idx / (2 * G * nz), yi = (idx / nz) % (2 * G), zi = idx % nz;
        uww_chunk_desc d;
        memset(&d, 0, sizeof(d));
        d.pos[0] = sp->sub_chunk[0] - G + xi;
        d.pos[1] = sp->sub_chunk[1] - G + yi;
        d.pos[2] = sz + zi;
        d.cells = cells;
        d.cell_offset = r * nc;
        d.sample_offset = r * ns;
        gen_out[r] = d;
    }
    counts[0] = ng;
    counts[1] = nr;
    free(gens);
    return UWW_OK;
}

/* ---- terrain.wgsl:26-59 at each vertex ---------------------------------------- */
static float smoothstep_c(float a, float b, float x)
{
    float t = (x - a) / (b - a);
    t = t < 0.f ? 0.f : (t > 1.f ? 1.f : t);
    return t * t * (3.f - 2.f * t);
}
static float clampf_c(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

int oracle_shade_vertices(const uww_camera_uniform* cam, const uww_vert_color* verts, uint32_t nv, float* clip,
                          float* rgb, float* dist_light)
{
    const float half_pi = 3.14159f / 2.0f;
    for (uint32_t v = 0; v < nv; ++v) {
        const float* p = verts[v].pos;
        for (int i = 0; i < 4; ++i) {
            float r = cam->view_proj[i] * p[0];
            r = r + cam->view_proj[4 + i] * p[1];
            r = r + cam->view_proj[8 + i] * p[2];
            clip[4 * v + i] = r + cam->view_proj[12 + i];
        }
        const v3 dv = {p[0] - cam->sub_pos[0], p[1] - cam->sub_pos[1], p[2] - cam->sub_pos[2]};
        const v3 f = {cam->sub_forward[0], cam->sub_forward[1], cam->sub_forward[2]};
        const float dist = sqrtf(dot3(dv, dv));
        const float cos_angle = dot3(dv, f) / (dist * sqrtf(dot3(f, f)));
        const float angle = acosf(cos_angle);
        const float light0 = cosf(angle * 3.0f) * (angle < half_pi ? 1.0f : 0.0f);
        const float light = smoothstep_c(0.f, 1.f, light0);
        const float min_dist_value = smoothstep_c(0.f, 20.f, clampf_c(dist, 0.f, 20.f));
        const float max_dist_value = smoothstep_c(0.f, 45.f, clampf_c(dist, 0.f, 45.f));
        const float dark = clampf_c(1.0f - light, max_dist_value, min_dist_value);
        for (int i = 0; i < 3; ++i) rgb[3 * v + i] = verts[v].color[i] * (1.0f - dark) + cam->fog_color[i] * dark;
        dist_light[2 * v] = dist;
        dist_light[2 * v + 1] = light;
    }
    return UWW_OK;
}
