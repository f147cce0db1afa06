/*
 * uww_oracle.h -- CPU oracle of the chunk-generation path.
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker; never by the product library.
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
double oracle_density64_full(const uww_params* p, const uint8_t* P, double wx, double wy, double wz,
                             double* grad);

#ifdef __cplusplus
}
#endif
#endif
