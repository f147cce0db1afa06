/*
 * uww_oracle.h -- CPU oracle of the chunk-generation path.
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py, to verify and time against; never by the product library.
 */
#ifndef UWW_ORACLE_H
#define UWW_ORACLE_H
#include <stdint.h>
#include "uww.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_F32 0            /* f32 in the GPU parity build's operation order     */
#define ORACLE_F64 1            /* reference semantics: f64 noise, f32 bias and mesh */
#define ORACLE_SEARCH_LINEAR 0  /* reference O(V) dedup search (chunk.rs:233)        */
#define ORACLE_SEARCH_HASHED 1  /* same result, hashed lookup                        */

void   oracle_perm(uint32_t seed, uint8_t P[256]);
/* samples_in (optional): build from these samples (at desc.sample_offset) instead of the noise */
int    oracle_build_chunks(const uww_params* p, int precision, int search, const uww_chunk_desc* chunks,
                           uint32_t n, const uww_mesh_out* out, int threads, const float* samples_in,
                           uint64_t samples_in_count);
int    oracle_sample_grid(const uww_params* p, int precision, const uww_chunk_desc* d, float* isos);
int    oracle_density_at(const uww_params* p, int precision, const float* xyz, uint32_t n, float* out,
                         float* grad);
int    oracle_perlin(uint32_t seed, int precision, const double* xyz, uint32_t n, double* out);
/* FP64 reference of the topology-frozen adjoint (uww_oracle_adjoint.c): loss
 * L = sum_v pos_grad[v] . p_v over the vertices named by (records, edge_ids),
 * its dL/dtheta (theta_grad, octaves + 5), dL/d(sample) (sample_grad, added
 * at desc.sample_offset) and the f64 positions (3 per vertex); any output but
 * loss may be NULL.  theta (octaves + 5 doubles) overrides the parameters'
 * amplitudes, frequency, offset and iso level when not NULL; samples_in
 * (doubles at desc.sample_offset) replaces the noise when not NULL.  dmax
 * (optional, octaves + 5) receives max |d rho / d theta_i| over the samples
 * evaluated (1 for the iso level): the scale of each parameter's effect.
 * pole (optional, octaves + 5) receives min over vertices of |D| / |dD/dtheta_i|,
 * D = rho_B - rho_A: how far theta_i can move before some edge degenerates
 * (t has a pole there), which bounds a meaningful finite-difference step. */
int    oracle_adjoint64(const uww_params* p, const double* theta, const uww_chunk_desc* chunks, uint32_t n,
                        const uww_chunk_record* records, const uint32_t* edge_ids, const float* pos_grad,
                        const double* samples_in, double* loss, double* theta_grad, double* sample_grad,
                        double* positions, double* dmax, double* pole);
/* uww_oracle_query.c: per-cell first index from the cases, and the boids'
 * wall-avoidance ray casts (nearest hit per ray, -1 when none). */
int    oracle_cell_tri_offsets(const uww_chunk_desc* chunks, uint32_t n, const uint8_t* cases, uint32_t* first);
int    oracle_ray_query(const uww_params* p, const uww_chunk_desc* chunks, uint32_t n, const uww_chunk_record* records,
                        const uww_vert_color* verts, const uint32_t* inds, const uint8_t* cases, const float* origins,
                        uint32_t nq, const float* dirs, uint32_t nrays, int32_t range, float* out);
int    oracle_schedule_chunks(const uww_params* p, const uww_schedule_params* sp, const uww_chunk_desc* known,
                              const uww_chunk_record* known_records, uint32_t n_known, uww_chunk_desc* gen_out,
                              uint32_t gen_cap, int32_t* render_out, uint32_t render_cap, uint32_t* counts);
int    oracle_shade_vertices(const uww_camera_uniform* cam, const uww_vert_color* verts, uint32_t nv, float* clip,
                             float* rgb, float* dist_light);
double oracle_density64_full(const uww_params* p, const uint8_t* P, double wx, double wy, double wz,
                             double* grad);

#ifdef __cplusplus
}
#endif
#endif
