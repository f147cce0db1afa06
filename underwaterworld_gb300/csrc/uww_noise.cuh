// uww_noise.cuh -- named-barrier helpers and the fast build's column noise,
// shared by the batched build (uww_build.cu) and the sampling kernel
// (uww_sample.cu).  Reference: perlin_util.rs:6-29 over the noise crate's
// perlin_3d (perlin_util.rs:13), sampled as Chunk::build_iso (chunk.rs:105-129).
#pragma once
#include <cuda_runtime.h>

#include "uww_internal.h"

namespace uww {
namespace {

// Named barriers: 0 = whole CTA, 1 = compute warps, 2 = ticket hand-off,
// 3 = offsets hand-off (2-3: compute warps + control warp).
constexpr int kBarCompute = 1;
constexpr int kBarTicket = 2;
constexpr int kBarOffsets = 3;

__device__ __forceinline__ void bar_arrive(int id, int count)
{
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__device__ __forceinline__ void bar_sync(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__device__ __forceinline__ int bar_or(int id, int count, int pred)
{
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.s32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.s32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(pred), "r"(id), "r"(count)
        : "memory");
    return r;
}

__device__ __forceinline__ int bar_and(int id, int count, int pred)
{
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.s32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.s32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(pred), "r"(id), "r"(count)
        : "memory");
    return r;
}

// ---------------------------------------------------------------------------
// Fast-build density grid, one compute thread per (x, y) column of samples.
//
// Along a column only z varies, and the z lattice cell, fraction and fade of
// every octave depend on z alone: they are tabulated once per chunk in shared
// memory, together with each octave's runs of consecutive samples that share
// a z lattice cell.  Per column and octave the x/y lattice coordinates,
// fades, partial hashes and bilinear weights are computed once; per run the
// corner gradients (from gp, the gradient of P[i]) of the run's two z lattice
// planes are reduced to the run's polynomial in dz:
//   A = g.xy . (d - o).xy and G = g.z per corner,
//   SA_c = sum_xy w A_xyc,  SG_c = sum_xy w G_xyc  (plane c = 0, 1),
//   n(dz) = al + be dz + fade(dz) (ga + de dz),
//   al = SA_0,  be = SG_0,  ga = SA_1 - SG_1 - SA_0,  de = SG_1 - SG_0,
// so a sample costs three FMAs plus its accumulate, and a run whose lower
// plane is the previous run's upper plane reads only four gradients.  Same Perlin/fBm maths as
// the parity build (trilinear interpolation == the k-polynomial) in a
// different operation order with FMA contraction.  The depth bias seeds the
// first octave; the early blank vote reads the last.  Returns whether any of
// this thread's samples is at or below the iso-level.  Every compute thread
// must call it.
// ---- arithmetic shared by every fast-build noise path ---------------------
// Only explicitly rounded operations (__fadd_rn, __fmul_rn, ...) and explicit
// fmaf: the compiler cannot contract them differently in different kernels,
// so the batched build and the sampling kernel produce the same samples.
__device__ __forceinline__ float fade_fma(float t)
{   // t^3 (t (6t - 15) + 10)
    return __fmul_rn(__fmul_rn(__fmul_rn(t, t), t), fmaf(t, fmaf(t, 6.f, -15.f), 10.f));
}

// noise-space amplitude scale of the octave sum: 2/sqrt(3), divided by the
// amplitude sum when normalised
__device__ __forceinline__ float fbm_norm(const DevParams& p)
{
    if (!p.normalize) return kPerlinScale;
    float mx = 0.f;
    for (int k = 0; k < p.octaves; ++k) mx = __fadd_rn(mx, p.amp[k]);
    return __fdiv_rn(kPerlinScale, mx);
}

// z-table entry of octave k at sample z: fraction, its fade, lattice cell
__device__ __forceinline__ void z_entry(const DevParams& p, int k, int z, float s, float zoff, float& dz, float& fd,
                                        int& cell)
{
    const float qz = __fmul_rn(fmaf((float)z, s, zoff), __fmul_rn(p.base_freq, p.mult[k]));
    const float fz = floorf(qz);
    dz = __fsub_rn(qz, fz);
    fd = fade_fma(dz);
    cell = (int)fz;
}

// depth bias at sample z
__device__ __forceinline__ float z_bias(const DevParams& p, int z, float s, int oz)
{
    const float wz = fmaf((float)z, s, (float)oz);
    if (p.bias_mode == UWW_BIAS_TERRACED) {
        const float adj = __fdiv_rn(__fmul_rn(__fmul_rn(__fadd_rn(wz, p.offset[2]), p.base_freq), p.bias_a), p.bias_b);
        return __fsub_rn(adj, fmodf(adj, p.bias_c));
    }
    if (p.bias_mode == UWW_BIAS_LINEAR) return __fmul_rn(p.bias_a, __fsub_rn(wz, p.bias_b));
    return 0.f;
}

// A bound on |fBm|.  Each octave's Perlin value is the trilinear blend, with
// weights W_c from the fade curve, of g_c . d_c over the cube's corners c,
// where every gradient g_c has two components of +-1 and one 0 and d_c is the
// offset from the corner; so |g_c . d_c| <= S_c = |dx|+|dy|+|dz| - min(|dx|,
// |dy|, |dz|) whatever the permutation, and |value| <= F = sum_c W_c S_c.  On
// a 201^3 grid of the unit cube max F = 1.0364; |grad F| <= 8.5 sqrt(3)
// (sum_c |dW_c/du| = 2 fade'(u) <= 3.75, S_c <= 2, |dS_c/du| <= 1), so
// between grid points F exceeds the grid maximum by at most
// 8.5 sqrt(3) * 0.005 sqrt(3) / 2 = 0.064: |value| <= 1.11 before the output
// scale (test_oracle.py recomputes both).  The fBm sums the octaves with
// weights amp_k * norm.
constexpr float kPerlinBound = 1.11f;

__device__ __forceinline__ float fbm_bound(const DevParams& p)
{
    float sa = 0.f;
    for (int k = 0; k < p.octaves; ++k) sa = __fadd_rn(sa, fabsf(p.amp[k]));
    return __fmul_rn(__fmul_rn(kPerlinBound, fabsf(fbm_norm(p))), sa);
}

// Whether the depth bias alone decides every sample of a chunk with N cells
// per edge at z offset oz: 1 when every sample is above the iso level (an
// early blank chunk), 2 when every sample is below it (every case 255), 0
// otherwise.  The margin covers f32 rounding and, for the terraced bias, a
// step of the staircase (the parity and fast builds may round the depth to
// either side of a step).  Every operation is explicitly rounded, so the
// planning kernel and the build kernel reach the same decision.
// B = fbm_bound(p) and s = chunk_size / N passed in (per-launch and per-LOD
// constants).
__device__ __forceinline__ int bias_decides_with(const DevParams& p, float B, float s, int N, int oz,
                                                 int* rank = nullptr)
{
    float lo = 3.0e38f, hi = -3.0e38f;
    bool ok = true;
    // the linear bias is monotonic in z: its ends suffice
    const int step = p.bias_mode == UWW_BIAS_TERRACED ? 1 : N;
    for (int z = 0; z <= N; z += step) {
        const float b = z_bias(p, z, s, oz);
        ok = ok && fabsf(b) < 1.0e30f;  // false for NaN too
        lo = fminf(lo, b);
        hi = fmaxf(hi, b);
    }
    const float iso = p.iso_level;
    if (!ok || !(B < 1.0e30f) || !(fabsf(iso) < 1.0e30f)) return 0;
    float m = __fmul_rn(1.0e-3f, __fadd_rn(__fadd_rn(1.f, B), fmaxf(fabsf(lo), fabsf(hi))));
    if (p.bias_mode == UWW_BIAS_TERRACED) m = __fadd_rn(m, fabsf(p.bias_c));
    if (__fsub_rn(__fsub_rn(lo, B), m) > iso) return 1;
    if (__fadd_rn(__fadd_rn(hi, B), m) < iso) return 2;
    if (rank) {
        // how far the bias range stays from the iso level, in eighths of the
        // reach B + m: 0 when it contains the iso level (such a chunk most
        // likely holds the surface, and meshing makes it the costliest)
        const float gap = lo > iso ? lo - iso : (hi < iso ? iso - hi : 0.f);
        *rank = min(7, (int)(8.f * gap / (B + m)));
    }
    return 0;
}

__device__ __forceinline__ int bias_decides(const DevParams& p, int N, int oz)
{
    return bias_decides_with(p, fbm_bound(p), __fdiv_rn((float)p.chunk_size, (float)N), N, oz);
}

// noise coordinate of a column: (i s + o + offset) f
__device__ __forceinline__ float column_coord(float i, float s, int o, float off, float f)
{
    return __fmul_rn(__fadd_rn(fmaf(i, s, (float)o), off), f);
}

// x/y part of one octave at one column: fractions, bilinear weights (times the
// octave's amplitude), and the hashes of the four xy lattice corners
struct ColumnOctave {
    float dx, dy, dx1, dy1, w00, w01, w10, w11;
    int h00, h01, h10, h11;
};

__device__ __forceinline__ ColumnOctave column_octave(const DevParams& p, const uint8_t* __restrict__ P, float nx,
                                                      float ny, int k, float norm)
{
    ColumnOctave c;
    const float m = p.mult[k], amp = __fmul_rn(p.amp[k], norm);
    const float qx = __fmul_rn(nx, m), qy = __fmul_rn(ny, m);
    const float fx = floorf(qx), fy = floorf(qy);
    const int ix = (int)fx, iy = (int)fy;
    c.dx = __fsub_rn(qx, fx);
    c.dy = __fsub_rn(qy, fy);
    c.dx1 = __fsub_rn(c.dx, 1.f);
    c.dy1 = __fsub_rn(c.dy, 1.f);
    const float a = fade_fma(c.dx), b = fade_fma(c.dy);
    const float a0 = __fmul_rn(amp, __fsub_rn(1.f, a)), a1 = __fmul_rn(amp, a);
    const float b0 = __fsub_rn(1.f, b);
    c.w00 = __fmul_rn(a0, b0);
    c.w10 = __fmul_rn(a1, b0);
    c.w01 = __fmul_rn(a0, b);
    c.w11 = __fmul_rn(a1, b);
    const int hx0 = P[ix & 255], hx1 = P[(ix + 1) & 255];
    c.h00 = P[hx0 ^ (iy & 255)];
    c.h01 = P[hx0 ^ ((iy + 1) & 255)];
    c.h10 = P[hx1 ^ (iy & 255)];
    c.h11 = P[hx1 ^ ((iy + 1) & 255)];
    return c;
}

// weighted face sums over the four xy corners of z lattice plane pl:
// SA = sum w (g.xy . (d - o).xy), SG = sum w g.z
__device__ __forceinline__ void column_face(const ColumnOctave& c, const float4* __restrict__ gp, int pl, float& SA,
                                            float& SG)
{
    const float4 g00 = gp[c.h00 ^ pl], g01 = gp[c.h01 ^ pl], g10 = gp[c.h10 ^ pl], g11 = gp[c.h11 ^ pl];
    SA = fmaf(c.w00, fmaf(g00.x, c.dx, __fmul_rn(g00.y, c.dy)),
              fmaf(c.w01, fmaf(g01.x, c.dx, __fmul_rn(g01.y, c.dy1)),
                   fmaf(c.w10, fmaf(g10.x, c.dx1, __fmul_rn(g10.y, c.dy)),
                        __fmul_rn(c.w11, fmaf(g11.x, c.dx1, __fmul_rn(g11.y, c.dy1))))));
    SG = fmaf(c.w00, g00.z, fmaf(c.w01, g01.z, fmaf(c.w10, g10.z, __fmul_rn(c.w11, g11.z))));
}

// a run's polynomial n(dz) = al + be dz + fade(dz) (ga + de dz) from the face
// sums of its lower (0) and upper (1) planes, and its value at one sample
struct RunPoly {
    float al, be, ga, de;
};
__device__ __forceinline__ RunPoly run_poly(float SA0, float SG0, float SA1, float SG1)
{
    return {SA0, SG0, __fsub_rn(__fsub_rn(SA1, SG1), SA0), __fsub_rn(SG1, SG0)};
}
__device__ __forceinline__ float run_value(const RunPoly& q, float2 t)
{
    return fmaf(t.y, fmaf(q.de, t.x, q.ga), fmaf(q.be, t.x, q.al));
}

struct ZTable {
    float2* dzc;      // [octave][z]: (dz, fade(dz))
    int2* runs;       // [octave][run]: (first z, z lattice cell)
    int* nruns;       // [octave]
    float* bias;      // [z]
    unsigned* rmask;  // [octave]: bit z set where a run starts (S <= 32)
};

__device__ __forceinline__ ZTable ztable_at(uint8_t* base, int S, int octaves)
{
    ZTable t;
    t.dzc = reinterpret_cast<float2*>(base);
    t.runs = reinterpret_cast<int2*>(base + (size_t)octaves * S * sizeof(float2));
    t.nruns = reinterpret_cast<int*>(base + (size_t)octaves * S * (sizeof(float2) + sizeof(int2)));
    t.bias = reinterpret_cast<float*>(base + (size_t)octaves * S * (sizeof(float2) + sizeof(int2)) +
                                      (size_t)octaves * sizeof(int));
    t.rmask = reinterpret_cast<unsigned*>(base + (size_t)octaves * S * (sizeof(float2) + sizeof(int2)) +
                                          (size_t)octaves * sizeof(int) + (size_t)S * sizeof(float));
    return t;
}

// The z tables of one chunk of S <= 32 samples per edge, one warp per octave:
// lane z computes its entry and its predecessor's lattice cell, a ballot
// marks the run starts, and each start is written to its run slot.  The same
// entries and runs as the serial compaction of sample_columns_fast.  Every
// compute thread calls it; the caller synchronises the compute warps after.
__device__ __forceinline__ void ztable_warps(const DevParams& p, const ZTable Z, int S, float s, float zoff, int oz,
                                             int ncomp)
{
    const int K = p.octaves, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = ncomp >> 5;
    for (int k = warp; k < K; k += nwarps) {
        float dz, fd, dzp, fdp;
        int cell, cellp;
        z_entry(p, k, lane, s, zoff, dz, fd, cell);
        z_entry(p, k, lane - 1, s, zoff, dzp, fdp, cellp);
        const bool on = lane < S;
        const unsigned m = __ballot_sync(0xffffffffu, on && (lane == 0 || cellp != cell));
        if (on) Z.dzc[k * S + lane] = make_float2(dz, fd);
        if ((m >> lane) & 1u) Z.runs[k * S + __popc(m & ((1u << lane) - 1u))] = make_int2(lane, cell);
        if (lane == 0) {
            Z.nruns[k] = __popc(m);
            Z.rmask[k] = m;
        }
    }
    for (int z = threadIdx.x; z < S; z += ncomp) Z.bias[z] = z_bias(p, z, s, oz);
}

// Settling a chunk early.  After the first octaves a chunk whose every
// partial sum stays above (below) the iso level by more than the remaining
// octaves can reach is blank (solid) whatever they add: its other octaves are
// not needed (its samples are not kept, so callers that write samples do not
// settle early).  The reach is kPerlinBound |norm| sum_{k' > k} |amp_k'| (see
// fbm_bound) and the margin covers f32 rounding as in bias_decides_with.
// Checked after octaves 0 .. kSettleChecks-1, in fBm of at least
// kSettleMinOctaves octaves (with fewer the checks' barriers cost more than
// the octaves they skip).
constexpr int kSettleChecks = 2;
constexpr int kSettleMinOctaves = 5;

__device__ __forceinline__ float fbm_reach_after(const DevParams& p, int k)
{
    float sa = 0.f;
    for (int j = k + 1; j < p.octaves; ++j) sa = __fadd_rn(sa, fabsf(p.amp[j]));
    return __fmul_rn(__fmul_rn(kPerlinBound, fabsf(fbm_norm(p))), sa);
}

// bit 0: partial sum v stays above the iso level whatever the reach R adds;
// bit 1: it stays below
__device__ __forceinline__ unsigned settled_bits(float v, float R, float iso)
{
    const float m = __fmul_rn(1.0e-3f, __fadd_rn(__fadd_rn(1.f, R), fabsf(v)));
    return (__fsub_rn(__fsub_rn(v, R), m) > iso ? 1u : 0u) | (__fadd_rn(__fadd_rn(v, R), m) < iso ? 2u : 0u);
}

// sample_columns_fast for chunks of S samples per edge (a compile-time S <=
// 32) in shared memory: each thread's column is accumulated in registers,
// over a fully unrolled z loop whose run starts are uniform branches, and
// written to rho once.  Operation for operation the arithmetic of
// sample_columns_fast (and of the sampling kernel), so the samples are the
// same bits.  Returns the same votes.  Every compute thread must call it.
template <int S>
__device__ __forceinline__ int sample_columns_reg(const DevParams& p, const uint8_t* __restrict__ P,
                                                  const float4* __restrict__ gp, const ZTable Z,
                                                  float* __restrict__ rho, int ox, int oy, int oz, int ncomp,
                                                  unsigned long long* masks = nullptr)
{
    constexpr int SS = S * S;
    const int K = p.octaves;
    const float s = __fdiv_rn((float)p.chunk_size, (float)(S - 1));
    const float bf = p.base_freq;
    const float norm = fbm_norm(p);
    const float zoff = __fadd_rn((float)oz, p.offset[2]);
    const float iso = p.iso_level;
    ztable_warps(p, Z, S, s, zoff, oz, ncomp);
    bar_sync(kBarCompute, ncomp);

    int inside = 0, outside = 0;
    for (int col = threadIdx.x; col < SS; col += ncomp) {
        const int x = col / S, y = col - x * S;
        const float nx = column_coord((float)x, s, ox, p.offset[0], bf);
        const float ny = column_coord((float)y, s, oy, p.offset[1], bf);
        float acc[S];
#pragma unroll
        for (int z = 0; z < S; ++z) acc[z] = Z.bias[z];
        for (int k = 0; k < K; ++k) {
            const ColumnOctave co = column_octave(p, P, nx, ny, k, norm);
            const unsigned rm = Z.rmask[k];
            const int2* runs = Z.runs + k * S;
            const float2* dzc = Z.dzc + k * S;
            float SA0 = 0.f, SG0 = 0.f, SA1 = 0.f, SG1 = 0.f;
            RunPoly q = {0.f, 0.f, 0.f, 0.f};
            int prev = 0, r = 0;
#pragma unroll
            for (int z = 0; z < S; ++z) {
                if (rm & (1u << z)) {  // the same for every column
                    const int c = runs[r++].y;
                    if (z > 0 && c == prev + 1) {
                        SA0 = SA1;
                        SG0 = SG1;
                    } else {
                        column_face(co, gp, c & 255, SA0, SG0);
                    }
                    column_face(co, gp, (c + 1) & 255, SA1, SG1);
                    prev = c;
                    q = run_poly(SA0, SG0, SA1, SG1);
                }
                acc[z] = __fadd_rn(run_value(q, dzc[z]), acc[z]);
            }
        }
        float* out = rho + col * S;
        unsigned below = 0;
#pragma unroll
        for (int z = 0; z < S; ++z) {
            out[z] = acc[z];
            inside |= !(acc[z] > iso);
            outside |= !(acc[z] < iso);
            below |= (unsigned)(acc[z] < iso) << z;
        }
        if (masks) masks[col] = below;
    }
    return inside | (outside << 1);
}

// The per-chunk z tables of S samples per edge (any S), shared by every
// column: entries by all compute threads, then each octave's cells compacted
// into runs by one thread.  Every compute thread calls it; it synchronises
// the compute warps before it returns.
__device__ __forceinline__ void ztable_serial(const DevParams& p, const ZTable Z, int S, float s, float zoff, int oz,
                                              int ncomp)
{
    const int K = p.octaves;
    for (int i = threadIdx.x; i < K * S; i += ncomp) {
        const int k = i / S, z = i - k * S;
        float dz, fd;
        int cell;
        z_entry(p, k, z, s, zoff, dz, fd, cell);
        Z.dzc[i] = make_float2(dz, fd);
        reinterpret_cast<int*>(Z.runs)[2 * i + 1] = cell;  // staged: cell of sample z
        if (k == 0) Z.bias[z] = z_bias(p, z, s, oz);
    }
    bar_sync(kBarCompute, ncomp);
    for (int k = threadIdx.x; k < K; k += ncomp) {
        int2* r = Z.runs + k * S;
        int n = 0, prev = 0;
        for (int z = 0; z < S; ++z) {
            const int iz = r[z].y;  // staged value; r[n] with n <= z is already consumed
            if (z == 0 || iz != prev) r[n++] = make_int2(z, iz);
            prev = iz;
        }
        Z.nruns[k] = n;
    }
    bar_sync(kBarCompute, ncomp);
}

// One octave of one column accumulated into out[0..S) (shared memory or a
// per-thread buffer), the operations of sample_columns_fast; on the last
// octave also the votes and the below-iso bits.
__device__ __forceinline__ void column_octave_runs(const DevParams& p, const uint8_t* __restrict__ P,
                                                   const float4* __restrict__ gp, const ZTable Z, int S, float nx,
                                                   float ny, float norm, int k, float* out, float iso, int& inside,
                                                   int& outside, unsigned long long& below)
{
    const int K = p.octaves;
    const ColumnOctave co = column_octave(p, P, nx, ny, k, norm);
    const float2* dzc = Z.dzc + k * S;
    const int2* runs = Z.runs + k * S;
    const int nr = Z.nruns[k];
    const bool first = k == 0, last = k == K - 1;
    // consecutive runs usually sit in consecutive z cells, whose shared
    // plane is then read once (the condition is the same for every column)
    float SA0 = 0.f, SG0 = 0.f, SA1 = 0.f, SG1 = 0.f;
    int prev = 0;
    for (int r = 0; r < nr; ++r) {
        const int2 run = runs[r];
        const int zb = run.x, ze = r + 1 < nr ? runs[r + 1].x : S;
        if (r > 0 && run.y == prev + 1) {
            SA0 = SA1;
            SG0 = SG1;
        } else {
            column_face(co, gp, run.y & 255, SA0, SG0);
        }
        column_face(co, gp, (run.y + 1) & 255, SA1, SG1);
        prev = run.y;
        const RunPoly q = run_poly(SA0, SG0, SA1, SG1);
#pragma unroll 2
        for (int z = zb; z < ze; ++z) {
            const float r0 = __fadd_rn(run_value(q, dzc[z]), first ? Z.bias[z] : out[z]);
            out[z] = r0;
            if (last) {
                inside |= !(r0 > iso);
                outside |= !(r0 < iso);  // a case bit stays clear
                below |= (unsigned long long)(r0 < iso) << (z & 63);
            }
        }
    }
}

// sample_columns_fast with rho in shared memory, for at most one column per
// compute thread (planes * S <= ncomp): the same samples, masks and votes.
// With settle it checks, after octaves 0 .. kSettleChecks-1, whether the
// slab has settled: then rho and masks are not complete and it returns the
// votes of a blank (2) or a solid (1) one.  Every compute thread must call it.
__device__ __forceinline__ int sample_columns_fast_settle(const DevParams& p, const uint8_t* __restrict__ P,
                                                          const float4* __restrict__ gp, const ZTable Z,
                                                          float* __restrict__ rho, int N, int ox, int oy, int oz,
                                                          int ncomp, unsigned long long* masks, int xlo, int planes,
                                                          bool settle)
{
    const int S = N + 1, SS = planes * S, K = p.octaves;
    const float s = __fdiv_rn((float)p.chunk_size, (float)N);
    const float bf = p.base_freq;
    const float norm = fbm_norm(p);
    const float zoff = __fadd_rn((float)oz, p.offset[2]);
    const float iso = p.iso_level;
    ztable_serial(p, Z, S, s, zoff, oz, ncomp);

    const int col = threadIdx.x;
    const bool has = col < SS;
    const int x = xlo + (has ? col / S : 0), y = has ? col - (col / S) * S : 0;
    const float nx = column_coord((float)x, s, ox, p.offset[0], bf);
    const float ny = column_coord((float)y, s, oy, p.offset[1], bf);
    float* out = rho + (has ? col : 0) * S;
    int inside = 0, outside = 0;
    unsigned long long below = 0ull;
    for (int k = 0; k < K; ++k) {
        if (has) column_octave_runs(p, P, gp, Z, S, nx, ny, norm, k, out, iso, inside, outside, below);
        if (settle && k < kSettleChecks && k + 1 < K) {
            const float R = fbm_reach_after(p, k);
            unsigned st = 3u;
            if (has)
                for (int z = 0; z < S; ++z) st &= settled_bits(out[z], R, iso);
            if (bar_and(kBarCompute, ncomp, (int)(st & 1u))) return 2;  // blank
            if (bar_and(kBarCompute, ncomp, (int)(st >> 1))) return 1;   // solid
        }
    }
    if (has && masks) masks[col] = below;
    return inside | (outside << 1);
}

// Returns bit 0: a sample of this thread's columns is not above the iso
// level (the early blank vote); bit 1: one is not below it (its corner bit in
// a cell's case stays clear).
// COLBUF: accumulate each column in a per-thread buffer (local memory, L1)
// and write it to rho once, for rho in global memory where an accumulate per
// sample and octave would be an L2 round trip each.
// masks (optional, at most 64 samples per column): per column the bits z
// with sample < iso level -- the columns' corner bits of every cell case, so
// the classification reads no samples.
// xlo, planes: the x planes xlo .. xlo + planes - 1 only (a slab of the
// chunk; rho and masks then hold those planes' columns); planes < 0: all.
template <bool COLBUF = false>
__device__ __forceinline__ int sample_columns_fast(const DevParams& p, const uint8_t* __restrict__ P,
                                                   const float4* __restrict__ gp, const ZTable Z,
                                                   float* __restrict__ rho, int N, int ox, int oy, int oz,
                                                   int ncomp, unsigned long long* masks = nullptr, int xlo = 0,
                                                   int planes = -1)
{
    const int S = N + 1, SS = (planes < 0 ? S : planes) * S, K = p.octaves;
    const float s = __fdiv_rn((float)p.chunk_size, (float)N);
    const float bf = p.base_freq;
    const float norm = fbm_norm(p);
    const float zoff = __fadd_rn((float)oz, p.offset[2]);
    const float iso = p.iso_level;

    ztable_serial(p, Z, S, s, zoff, oz, ncomp);

    int inside = 0, outside = 0;
    for (int col = threadIdx.x; col < SS; col += ncomp) {
        const int x = xlo + col / S, y = col - (col / S) * S;
        float colbuf[COLBUF ? UWW_MAX_CELLS + 1 : 1];
        unsigned long long below = 0ull;
        float* out = COLBUF ? colbuf : rho + col * S;
        const float nx = column_coord((float)x, s, ox, p.offset[0], bf);
        const float ny = column_coord((float)y, s, oy, p.offset[1], bf);
        for (int k = 0; k < K; ++k) {
            const ColumnOctave co = column_octave(p, P, nx, ny, k, norm);
            const float2* dzc = Z.dzc + k * S;
            const int2* runs = Z.runs + k * S;
            const int nr = Z.nruns[k];
            const bool first = k == 0, last = k == K - 1;
            // consecutive runs usually sit in consecutive z cells, whose shared
            // plane is then read once (the condition is the same for every column)
            float SA0 = 0.f, SG0 = 0.f, SA1 = 0.f, SG1 = 0.f;
            int prev = 0;
            for (int r = 0; r < nr; ++r) {
                const int2 run = runs[r];
                const int zb = run.x, ze = r + 1 < nr ? runs[r + 1].x : S;
                if (r > 0 && run.y == prev + 1) {
                    SA0 = SA1;
                    SG0 = SG1;
                } else {
                    column_face(co, gp, run.y & 255, SA0, SG0);
                }
                column_face(co, gp, (run.y + 1) & 255, SA1, SG1);
                prev = run.y;
                const RunPoly q = run_poly(SA0, SG0, SA1, SG1);
#pragma unroll 2
                for (int z = zb; z < ze; ++z) {
                    const float r0 = __fadd_rn(run_value(q, dzc[z]), first ? Z.bias[z] : out[z]);
                    out[z] = r0;
                    if (last) {
                        inside |= !(r0 > iso);
                        outside |= !(r0 < iso);  // a case bit stays clear
                        if (!COLBUF) below |= (unsigned long long)(r0 < iso) << (z & 63);
                    }
                }
            }
        }
        if (COLBUF) {
            float* dst = rho + col * S;
            unsigned long long m = 0ull;
            for (int z = 0; z < S; ++z) {
                dst[z] = colbuf[z];
                m |= (unsigned long long)(colbuf[z] < iso) << (z & 63);
            }
            if (masks) masks[col] = m;
        } else if (masks) {
            masks[col] = below;
        }
    }
    return inside | (outside << 1);
}


}  // namespace
}  // namespace uww
