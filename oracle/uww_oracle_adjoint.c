/*
 * uww_oracle_adjoint.c -- FP64 CPU reference of the topology-frozen adjoint
 * (uww_forward / uww_backward of libuww_gb300.so).
 * TEST INFRASTRUCTURE ONLY: the product never links this file.
 *
 * The reference has no derivatives; this restates, in f64, the quantity the
 * GPU differentiates.  Each vertex v lies on the grid edge from sample A to
 * sample B of its chunk (the edge id the forward recorded):
 *     t_v = (iso - rho_A) / (rho_B - rho_A),   p_v = P_A + t_v (P_B - P_A) + origin,
 * with rho the density of perlin_util.rs:6-29 (fBm of the noise crate's
 * perlin_3d plus the depth bias) at the sample's world position
 * (i * SIZE_SCALE + origin, chunk.rs:105-129 with SIZE_SCALE the f32
 * chunk_size / cells widened), and L = sum_v c_v . p_v.
 * theta = (per-octave amplitudes, base frequency, world offset xyz, iso).
 * Derivatives are analytic (chain rule through t, fBm and each Perlin
 * octave's gradient); finite differences of L in theta use the same
 * function with theta perturbed.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "uww.h"
#include "uww_oracle.h"

/* only the Perlin core and the octave tables are used here */
#pragma GCC diagnostic ignored "-Wunused-function"
#define REAL double
#define SUFFIX _f64
#define FLOOR floor
#include "oracle_noise.inc"
#undef REAL

typedef struct {
    const uww_params* p;
    uint8_t P[256];
    int K;
    double mult[UWW_MAX_OCTAVES];
    double amp[UWW_MAX_OCTAVES];
    double f, off[3], iso;
} adj_world;

/* density at world w and, if d, its theta derivatives d[0..K-1] (amplitudes),
 * d[K] (frequency), d[K+1..K+3] (offset). */
static double density_theta64(const adj_world* w, const double wp[3], double* d)
{
    const uww_params* p = w->p;
    const int K = w->K;
    double u[3], nn[3];
    for (int j = 0; j < 3; ++j) {
        u[j] = wp[j] + w->off[j];
        nn[j] = u[j] * w->f;
    }
    double total = 0, maxv = 0, g[3] = {0, 0, 0}, v[UWW_MAX_OCTAVES];
    for (int k = 0; k < K; ++k) {
        double gk[3];
        v[k] = perlin_f64(w->P, nn[0] * w->mult[k], nn[1] * w->mult[k], nn[2] * w->mult[k], d ? gk : NULL);
        total += w->amp[k] * v[k];
        maxv += w->amp[k];
        if (d)
            for (int j = 0; j < 3; ++j) g[j] += w->amp[k] * w->mult[k] * gk[j];
    }
    double F = total;
    if (p->normalize) {
        F = total / maxv;
        if (d) {
            for (int k = 0; k < K; ++k) d[k] = (v[k] - F) / maxv;
            for (int j = 0; j < 3; ++j) g[j] /= maxv;
        }
    } else if (d) {
        for (int k = 0; k < K; ++k) d[k] = v[k];
    }
    if (d) {
        d[K] = g[0] * u[0] + g[1] * u[1] + g[2] * u[2];
        for (int j = 0; j < 3; ++j) d[K + 1 + j] = g[j] * w->f;
    }
    if (p->bias_mode == UWW_BIAS_TERRACED) {
        const double adj = nn[2] * (double)p->bias_a / (double)p->bias_b;
        return adj + F - fmod(adj, (double)p->bias_c);
    }
    if (p->bias_mode == UWW_BIAS_LINEAR) return F + (double)p->bias_a * (wp[2] - (double)p->bias_b);
    return F;
}

int oracle_adjoint64(const uww_params* p, const double* theta, const uww_chunk_desc* chunks, uint32_t n,
                     const uww_chunk_record* records, const uint32_t* edge_ids, const float* pos_grad,
                     const double* samples_in, double* loss, double* theta_grad, double* sample_grad,
                     double* positions, double* dmax, double* pole)
{
    if (!p || !chunks || !records || !edge_ids || !pos_grad || !loss) return UWW_ERR_INVALID_ARG;
    adj_world w;
    memset(&w, 0, sizeof(w));
    w.p = p;
    w.K = (int)p->octaves;
    if (w.K < 1 || w.K > UWW_MAX_OCTAVES) return UWW_ERR_INVALID_ARG;
    oracle_perm(p->seed, w.P);
    octave_tables_f64(p, w.mult, w.amp);
    w.f = p->base_freq;
    for (int j = 0; j < 3; ++j) w.off[j] = p->offset[j];
    w.iso = p->iso_level;
    if (theta) {
        for (int k = 0; k < w.K; ++k) w.amp[k] = theta[k];
        w.f = theta[w.K];
        for (int j = 0; j < 3; ++j) w.off[j] = theta[w.K + 1 + j];
        w.iso = theta[w.K + 4];
    }
    const int NT = w.K + 5;
    double L = 0;
    if (theta_grad)
        for (int j = 0; j < NT; ++j) theta_grad[j] = 0;
    if (dmax)
        for (int j = 0; j < NT; ++j) dmax[j] = j == NT - 1 ? 1.0 : 0.0;
    if (pole)
        for (int j = 0; j < NT; ++j) pole[j] = INFINITY;
    double dA[UWW_MAX_OCTAVES + 4], dB[UWW_MAX_OCTAVES + 4];
    for (uint32_t c = 0; c < n; ++c) {
        const uww_chunk_record* r = &records[c];
        if (!(r->flags & UWW_CHUNK_HAS_MESH) || (r->flags & UWW_CHUNK_OVERFLOW)) continue;
        const uww_chunk_desc* d = &chunks[c];
        const int N = (int)d->cells, S = N + 1;
        if (N < 1 || N > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
        const double s = (double)((float)p->chunk_size / (float)N);
        const double org[3] = {(double)d->pos[0] * p->chunk_size, (double)d->pos[1] * p->chunk_size,
                               (double)d->pos[2] * p->chunk_size};
        for (uint32_t v = 0; v < r->num_verts; ++v) {
            const uint32_t gid = r->vert_offset + v;
            const uint32_t e = edge_ids[gid], sa = e >> 3, dir = e & 7u;
            int a[3] = {(int)(sa / (uint32_t)(S * S)), (int)((sa / (uint32_t)S) % (uint32_t)S), (int)(sa % (uint32_t)S)};
            if (sa >= (uint32_t)(S * S * S) || dir > 5u) return UWW_ERR_INVALID_ARG;
            const int axis = (int)(dir >> 1);
            int b[3] = {a[0], a[1], a[2]};
            b[axis] += (dir & 1u) ? -1 : 1;
            if (b[axis] < 0 || b[axis] >= S) return UWW_ERR_INVALID_ARG;
            const uint32_t sb = (uint32_t)((b[0] * S + b[1]) * S + b[2]);
            double PA[3], PB[3], wa[3], wb[3];
            for (int j = 0; j < 3; ++j) {
                PA[j] = a[j] * s;
                PB[j] = b[j] * s;
                wa[j] = PA[j] + org[j];
                wb[j] = PB[j] + org[j];
            }
            const int want_d = (theta_grad || dmax || pole) && !samples_in;
            double ra, rb;
            if (samples_in) {
                ra = samples_in[d->sample_offset + sa];
                rb = samples_in[d->sample_offset + sb];
            } else {
                ra = density_theta64(&w, wa, want_d ? dA : NULL);
                rb = density_theta64(&w, wb, want_d ? dB : NULL);
            }
            if (dmax && want_d)
                for (int j = 0; j < w.K + 4; ++j) {
                    if (fabs(dA[j]) > dmax[j]) dmax[j] = fabs(dA[j]);
                    if (fabs(dB[j]) > dmax[j]) dmax[j] = fabs(dB[j]);
                }
            const double D = rb - ra;
            if (pole && want_d)
                for (int j = 0; j < w.K + 4; ++j) {
                    const double dd = fabs(dB[j] - dA[j]);
                    if (dd > 0 && fabs(D) / dd < pole[j]) pole[j] = fabs(D) / dd;
                }
            if (D == 0) continue;
            const double t = (w.iso - ra) / D;
            const float* cv = pos_grad + 3 * (size_t)gid;
            for (int j = 0; j < 3; ++j) {
                const double pj = PA[j] + t * (PB[j] - PA[j]) + org[j];
                L += (double)cv[j] * pj;
                if (positions) positions[3 * (size_t)gid + j] = pj;
            }
            const double dLdt = (double)cv[axis] * (PB[axis] - PA[axis]);
            const double gA = dLdt * (t - 1) / D, gB = -dLdt * t / D;
            if (theta_grad) {
                if (!samples_in)
                    for (int j = 0; j < w.K + 4; ++j) theta_grad[j] += gA * dA[j] + gB * dB[j];
                theta_grad[w.K + 4] += dLdt / D;
            }
            if (sample_grad) {
                sample_grad[d->sample_offset + sa] += gA;
                sample_grad[d->sample_offset + sb] += gB;
            }
        }
    }
    *loss = L;
    return UWW_OK;
}
