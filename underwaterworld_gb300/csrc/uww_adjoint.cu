// uww_adjoint.cu -- topology-frozen adjoint of the chunk build, and the
// heightmap loss of the terrain-fitting loop.  No counterpart in the
// reference, which has no derivatives; the forward it differentiates is the
// mesher of chunk.rs:135-264 over the density of perlin_util.rs:6-29.
//
// A vertex lies on the grid edge from sample A to sample B (the forward's
// interpolation order):
//     t = (iso - rho_A) / (rho_B - rho_A),   p = P_A + t (P_B - P_A) + origin,
// with P_A, P_B the samples' chunk-local positions, which do not depend on
// theta.  For a loss L(p) with cotangent c = dL/dp and D = rho_B - rho_A:
//     dL/dt     = c . (P_B - P_A)
//     dL/drho_A = dL/dt (t - 1) / D,   dL/drho_B = -dL/dt t / D,
//     dL/diso  += dL/dt / D.
// The density's parameter derivatives at a world point w, with
// u = w + offset, n = u * f and per-octave Perlin values v_k at n * m_k:
//     F = sum_k a_k v_k  (divided by S = sum_k a_k when normalised),
//     dF/da_k = v_k (or (v_k - F) / S),
//     dF/dn   = sum_k a_k m_k grad v_k (or / S),
//     dF/df   = dF/dn . u,    dF/doffset = dF/dn * f.
// The depth bias does not depend on theta (linear) or has zero derivative
// almost everywhere (terraced: adj - fmod(adj, c) is piecewise constant).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "uww_internal.h"

namespace uww {
namespace {

constexpr int kBwdThreads = 256;

// Density at a world point and its theta derivatives: d[k] = d/da_k for
// k < KMAX, d[KMAX] = d/df, d[KMAX+1..3] = d/doffset.  The value is computed
// in the same operation order as density<O, false>, so in the parity build
// it equals the forward's sample bit for bit.
template <class O, int KMAX>
__device__ __forceinline__ float density_theta(const DevParams& p, const uint8_t* P, float wx, float wy, float wz,
                                               float (&d)[KMAX + 4])
{
    const float ux = O::add(wx, p.offset[0]), uy = O::add(wy, p.offset[1]), uz = O::add(wz, p.offset[2]);
    const float f = p.base_freq;
    const float nx = O::mul(ux, f), ny = O::mul(uy, f), nz = O::mul(uz, f);
    float total = 0.f, maxv = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    float v[KMAX];
#pragma unroll
    for (int k = 0; k < KMAX; ++k) {
        v[k] = 0.f;
        if (k < p.octaves) {
            const float m = p.mult[k], am = p.amp[k];
            float g[3];
            v[k] = perlin<O, true>(P, O::mul(nx, m), O::mul(ny, m), O::mul(nz, m), g);
            total = O::add(total, O::mul(v[k], am));
            maxv = O::add(maxv, am);
            gx = O::add(gx, O::mul(O::mul(g[0], am), m));
            gy = O::add(gy, O::mul(O::mul(g[1], am), m));
            gz = O::add(gz, O::mul(O::mul(g[2], am), m));
        }
    }
    float F = total;
    if (p.normalize) {
        F = __fdiv_rn(total, maxv);
        const float inv = __fdiv_rn(1.f, maxv);
#pragma unroll
        for (int k = 0; k < KMAX; ++k) d[k] = k < p.octaves ? O::mul(O::sub(v[k], F), inv) : 0.f;
        gx = O::mul(gx, inv);
        gy = O::mul(gy, inv);
        gz = O::mul(gz, inv);
    } else {
#pragma unroll
        for (int k = 0; k < KMAX; ++k) d[k] = v[k];
    }
    d[KMAX] = O::add(O::add(O::mul(gx, ux), O::mul(gy, uy)), O::mul(gz, uz));
    d[KMAX + 1] = O::mul(gx, f);
    d[KMAX + 2] = O::mul(gy, f);
    d[KMAX + 3] = O::mul(gz, f);
    if (p.bias_mode == UWW_BIAS_TERRACED) {
        const float adj = __fdiv_rn(O::mul(nz, p.bias_a), p.bias_b);
        return O::sub(O::add(adj, F), fmodf(adj, p.bias_c));
    }
    if (p.bias_mode == UWW_BIAS_LINEAR) return O::add(F, O::mul(p.bias_a, O::sub(wz, p.bias_b)));
    return F;
}

// ---- compensated (float-float) density for the backward --------------------
// t = (iso - rho_A) / (rho_B - rho_A) makes dL/drho scale as 1/D: on edges
// whose two samples are both near the iso-level, an f32 density error of
// ~1e-7 would move the gradient by percents.  The backward therefore
// evaluates the two densities as unevaluated sums hi + lo of two floats
// (Dekker's and Knuth's error-free transformations: TwoSum, and TwoProd by
// FMA, as in the double-double arithmetic of Hida, Li and Bailey), which
// carries about 44 significant bits; no FP64 instruction is used.
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_norm(float s, float e)
{   // fast two-sum, |s| >= |e|
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ff ff_add(ff x, ff y)
{
    const ff s = two_sum(x.hi, y.hi);
    return ff_norm(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ ff ff_add(ff x, float y)
{
    const ff s = two_sum(x.hi, y);
    return ff_norm(s.hi, __fadd_rn(s.lo, x.lo));
}
__device__ __forceinline__ ff ff_neg(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }
__device__ __forceinline__ ff ff_mul(ff x, ff y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    const float e = __fmaf_rn(x.hi, y.hi, -p);
    return ff_norm(p, __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, e)));
}
__device__ __forceinline__ ff ff_mul(ff x, float y)
{
    const float p = __fmul_rn(x.hi, y);
    const float e = __fmaf_rn(x.hi, y, -p);
    return ff_norm(p, __fmaf_rn(x.lo, y, e));
}
__device__ __forceinline__ ff ff_div(ff x, ff y)
{   // one correction step of the quotient
    const float q = __fdiv_rn(x.hi, y.hi);
    const ff r = ff_sub(x, ff_mul(y, q));
    return ff_norm(q, __fdiv_rn(r.hi, y.hi));
}
__device__ __forceinline__ ff ff_of(float a) { return {a, 0.f}; }

// 2/sqrt(3) as hi + lo (both parts are compile-time constants)
constexpr float kScaleHi = 1.1547005383792515f;
constexpr float kScaleLo = (float)(1.1547005383792515 - (double)kScaleHi);

__device__ __forceinline__ ff ff_grad_dot(int h, ff x, ff y, ff z)
{
    const unsigned c = (unsigned)(kGradCode >> ((h & 15) * 4)) & 15u;
    ff u = (c & 1u) ? y : x;
    ff v = (c & 4u) ? z : y;
    if (c & 2u) u = ff_neg(u);
    if (c & 8u) v = ff_neg(v);
    return ff_add(u, v);
}

__device__ __forceinline__ ff ff_fade(ff t)
{   // t^3 (t (6t - 15) + 10)
    const ff inner = ff_add(ff_mul(t, ff_add(ff_mul(t, 6.f), -15.f)), 10.f);
    return ff_mul(ff_mul(ff_mul(t, t), t), inner);
}

__device__ ff ff_perlin(const uint8_t* P, ff px, ff py, ff pz)
{
    // floor of hi + lo
    float fx = floorf(px.hi), fy = floorf(py.hi), fz = floorf(pz.hi);
    if (px.hi == fx && px.lo < 0.f) fx -= 1.f;
    if (py.hi == fy && py.lo < 0.f) fy -= 1.f;
    if (pz.hi == fz && pz.lo < 0.f) fz -= 1.f;
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    const ff dx = ff_add(px, -fx), dy = ff_add(py, -fy), dz = ff_add(pz, -fz);
    const ff dx1 = ff_add(dx, -1.f), dy1 = ff_add(dy, -1.f), dz1 = ff_add(dz, -1.f);
    const int a0 = P[ix & 255], a1 = P[(ix + 1) & 255];
    const int b00 = P[a0 ^ (iy & 255)], b01 = P[a0 ^ ((iy + 1) & 255)];
    const int b10 = P[a1 ^ (iy & 255)], b11 = P[a1 ^ ((iy + 1) & 255)];
    const int z0 = iz & 255, z1 = (iz + 1) & 255;
    const ff g000 = ff_grad_dot(P[b00 ^ z0], dx, dy, dz);
    const ff g100 = ff_grad_dot(P[b10 ^ z0], dx1, dy, dz);
    const ff g010 = ff_grad_dot(P[b01 ^ z0], dx, dy1, dz);
    const ff g110 = ff_grad_dot(P[b11 ^ z0], dx1, dy1, dz);
    const ff g001 = ff_grad_dot(P[b00 ^ z1], dx, dy, dz1);
    const ff g101 = ff_grad_dot(P[b10 ^ z1], dx1, dy, dz1);
    const ff g011 = ff_grad_dot(P[b01 ^ z1], dx, dy1, dz1);
    const ff g111 = ff_grad_dot(P[b11 ^ z1], dx1, dy1, dz1);
    const ff a = ff_fade(dx), b = ff_fade(dy), c = ff_fade(dz);
    // trilinear interpolation as lerps: along x, then y, then z
    auto lerp = [](ff t, ff u, ff v) { return ff_add(u, ff_mul(t, ff_sub(v, u))); };
    const ff x00 = lerp(a, g000, g100), x10 = lerp(a, g010, g110);
    const ff x01 = lerp(a, g001, g101), x11 = lerp(a, g011, g111);
    const ff y0 = lerp(b, x00, x10), y1 = lerp(b, x01, x11);
    return ff_mul(lerp(c, y0, y1), ff{kScaleHi, kScaleLo});
}

// The density at sample (x, y, z) of a chunk at origin o with cell size s,
// in float-float: world = x s + o exactly, then the same fBm and bias as
// density<O, false> (perlin_util.rs:6-29).
__device__ ff density_ff(const DevParams& p, const uint8_t* P, int x, int y, int z, float s, float ox, float oy,
                         float oz)
{
    ff w[3];
    const int ijk[3] = {x, y, z};
    const float org[3] = {ox, oy, oz};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const float pr = __fmul_rn((float)ijk[j], s);
        const ff prod = {pr, __fmaf_rn((float)ijk[j], s, -pr)};
        w[j] = ff_add(prod, org[j]);
    }
    ff n[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) n[j] = ff_mul(ff_add(w[j], p.offset[j]), p.base_freq);
    ff total = ff_of(0.f), maxv = ff_of(0.f);
    for (int k = 0; k < p.octaves; ++k) {
        const float m = p.mult[k];
        const ff v = ff_perlin(P, ff_mul(n[0], m), ff_mul(n[1], m), ff_mul(n[2], m));
        total = ff_add(total, ff_mul(v, p.amp[k]));
        maxv = ff_add(maxv, p.amp[k]);
    }
    const ff F = p.normalize ? ff_div(total, maxv) : total;
    if (p.bias_mode == UWW_BIAS_TERRACED) {
        // the terrace value adj - fmod(adj, c) is a multiple of c, computed
        // exactly as the forward computes it
        const float nz = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn((float)z, s), oz), p.offset[2]), p.base_freq);
        const float adj = __fdiv_rn(__fmul_rn(nz, p.bias_a), p.bias_b);
        return ff_add(F, __fsub_rn(adj, fmodf(adj, p.bias_c)));
    }
    if (p.bias_mode == UWW_BIAS_LINEAR) return ff_add(F, ff_mul(ff_add(w[2], -p.bias_b), p.bias_a));
    return F;
}

struct AdjointArgs {
    const uww_chunk_desc* chunks;
    const uww_chunk_record* records;
    const uint32_t* edge_ids;
    const float* pos_grad;           // [vert][3]
    float* sample_grad;              // optional, zeroed by the host
    unsigned long long sample_capacity;
    float* part;                     // [grid][KMAX + 5] per-CTA partials
    unsigned int* counter;           // zero at launch; the last CTA resets it
    float* theta_grad;               // [octaves + 5]
    uint32_t n;
    uint32_t max_cells;
};

template <int NV>
__device__ __forceinline__ void block_sum(float (&v)[NV], float (*red)[NV])
{
    // butterfly within each warp, then warps in a fixed order: deterministic
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < NV; ++j) red[warp][j] = v[j];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            float s = red[0][j];
            for (int w = 1; w < kBwdThreads / 32; ++w) s += red[w][j];
            v[j] = s;
        }
}

// Vertex-parallel over the batch: thread t of CTA b takes vertices
// b T + t, b T + t + G T, ... (T threads, G CTAs: a fixed assignment, so the
// sums below are deterministic), finds each vertex's chunk by binary search
// over the records' vertex offsets, recomputes the density and its theta
// derivatives at the edge's two corners, forms dL/drho_A, dL/drho_B and
// dL/diso, and accumulates dL/dtheta.  Per-CTA partials; the last CTA to
// finish reduces them in CTA order.  (One CTA per chunk left the densest
// chunks' CTAs as the tail of the launch.)
template <class O, int KMAX>
__global__ void __launch_bounds__(kBwdThreads) backward_kernel(const DevParams p, const AdjointArgs a)
{
    constexpr int NV = KMAX + 5;
    __shared__ __align__(16) uint8_t P[256];
    __shared__ float red[kBwdThreads / 32][NV];
    __shared__ unsigned int last;
    for (int i = threadIdx.x; i < 256; i += kBwdThreads) P[i] = p.perm[i];
    __syncthreads();

    float acc[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] = 0.f;
    float bad = 0.f;

    // the batch's vertices: the last chunk's inclusive prefix
    const uww_chunk_record rl = a.records[a.n - 1];
    const uint32_t V = rl.vert_offset + rl.num_verts;
    for (uint32_t gid = blockIdx.x * kBwdThreads + threadIdx.x; gid < V; gid += gridDim.x * kBwdThreads) {
        // its chunk: the last one whose first vertex is at or before it
        uint32_t c = 0, len = a.n;
        while (len > 1) {
            const uint32_t h = len >> 1;
            if (__ldg(&a.records[c + h].vert_offset) <= gid) c += h;
            len -= h;
        }
        const uww_chunk_record r = a.records[c];
        const uww_chunk_desc d = a.chunks[c];
        const bool use = (r.flags & UWW_CHUNK_HAS_MESH) && !(r.flags & UWW_CHUNK_OVERFLOW) && d.cells >= 1 &&
                         d.cells <= a.max_cells && gid - r.vert_offset < r.num_verts;
        if (!use) continue;
        const int N = (int)d.cells, S = N + 1;
        const uint32_t S3 = (uint32_t)S * S * S;
        const float s = __fdiv_rn((float)p.chunk_size, (float)N);
        const float ox = (float)(d.pos[0] * p.chunk_size), oy = (float)(d.pos[1] * p.chunk_size),
                    oz = (float)(d.pos[2] * p.chunk_size);
        const float iso = p.iso_level;
        const bool sg = a.sample_grad && (unsigned long long)d.sample_offset + S3 <= a.sample_capacity;
        {
            const uint32_t e = a.edge_ids[gid];
            const uint32_t sa = e >> 3, dir = e & 7u;
            const int xa = (int)(sa / (uint32_t)(S * S)), ya = (int)((sa / (uint32_t)S) % (uint32_t)S),
                      za = (int)(sa % (uint32_t)S);
            const int axis = (int)(dir >> 1), step = (dir & 1u) ? -1 : 1;
            const int xb = xa + (axis == 0 ? step : 0), yb = ya + (axis == 1 ? step : 0), zb = za + (axis == 2 ? step : 0);
            if (sa >= S3 || dir > 5u || xb < 0 || xb >= S || yb < 0 || yb >= S || zb < 0 || zb >= S) {
                bad = 1.f;
                continue;
            }
            // theta derivatives of the two densities in f32 ...
            float dA[KMAX + 4], dB[KMAX + 4];
            density_theta<O, KMAX>(p, P, O::add(O::mul((float)xa, s), ox), O::add(O::mul((float)ya, s), oy),
                                   O::add(O::mul((float)za, s), oz), dA);
            density_theta<O, KMAX>(p, P, O::add(O::mul((float)xb, s), ox), O::add(O::mul((float)yb, s), oy),
                                   O::add(O::mul((float)zb, s), oz), dB);
            // ... and their values in float-float, so that D and iso - rho_A
            // keep their relative accuracy on nearly degenerate edges
            const ff ra = density_ff(p, P, xa, ya, za, s, ox, oy, oz);
            const ff rb = density_ff(p, P, xb, yb, zb, s, ox, oy, oz);
            const float D = ff_sub(rb, ra).hi;
            if (D == 0.f) continue;
            const float t = __fdiv_rn(ff_sub(ff_of(iso), ra).hi, D);
            const int ia = axis == 0 ? xa : axis == 1 ? ya : za, ib = axis == 0 ? xb : axis == 1 ? yb : zb;
            const float dpdt = O::sub(O::mul((float)ib, s), O::mul((float)ia, s));
            const float dLdt = O::mul(a.pos_grad[3 * (size_t)gid + axis], dpdt);
            const float invD = __fdiv_rn(1.f, D);
            const float gA = O::mul(O::mul(dLdt, O::sub(t, 1.f)), invD);
            const float gB = -O::mul(O::mul(dLdt, t), invD);
#pragma unroll
            for (int j = 0; j < KMAX + 4; ++j) acc[j] = O::add(acc[j], O::add(O::mul(gA, dA[j]), O::mul(gB, dB[j])));
            acc[KMAX + 4] = O::add(acc[KMAX + 4], O::mul(dLdt, invD));
            if (sg) {
                const uint32_t sb = (uint32_t)((xb * S + yb) * S + zb);
                atomicAdd(a.sample_grad + d.sample_offset + sa, gA);
                atomicAdd(a.sample_grad + d.sample_offset + sb, gB);
            }
        }
    }
    // an edge id outside its chunk poisons the result instead of being dropped
    if (__syncthreads_or(bad != 0.f))
#pragma unroll
        for (int j = 0; j < NV; ++j) acc[j] = __int_as_float(0x7fc00000);
    block_sum<NV>(acc, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) a.part[(size_t)blockIdx.x * NV + j] = acc[j];
        __threadfence();
        last = atomicAdd(a.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // final reduction: thread i sums the partials of CTAs i, i + 256, ... in
    // order, then the block sum combines the threads in a fixed order
    float tot[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) tot[j] = 0.f;
    for (uint32_t k = threadIdx.x; k < gridDim.x; k += kBwdThreads)
#pragma unroll
        for (int j = 0; j < NV; ++j) tot[j] += __ldcg(a.part + (size_t)k * NV + j);
    __syncthreads();
    block_sum<NV>(tot, red);
    if (threadIdx.x == 0) {
        const int K = p.octaves;
        for (int k = 0; k < K; ++k) a.theta_grad[k] = tot[k];
        for (int j = 0; j < 5; ++j) a.theta_grad[K + j] = tot[KMAX + j];
        *a.counter = 0u;
    }
}

// ---- heightmap loss --------------------------------------------------------
// Column c = (floor((x - x0) / w), floor((y - y0) / w)); over the columns
// holding at least one vertex, L = sum (mean z - target)^2 / (cols_x cols_y).
// Deterministic: each column's heights are summed in 2^-16 fixed point with
// integer atomics (their order does not change the sum), and the loss is
// reduced over the columns in a fixed order by one CTA, so a terrain-fitting
// run repeats exactly.
constexpr double kHeightFix = 65536.0;  // fixed-point scale of the column sums

struct HeightArgs {
    const uww_vert_color* verts;
    const unsigned long long* totals;   // totals[0] = vertex count
    uint32_t vert_capacity;
    float x0, y0, inv_w;
    uint32_t cols_x, cols_y;
    const float* target;
    long long* sum_z;                   // [cols] sum of z * kHeightFix, rounded per vertex
    unsigned long long* count;          // [cols]
    float* pos_grad;
    float* loss;
};

__device__ __forceinline__ float column_mean(const HeightArgs& h, int c)
{
    return (float)((double)h.sum_z[c] / kHeightFix / (double)h.count[c]);
}

__device__ __forceinline__ int column_of(const HeightArgs& h, float x, float y)
{
    const int cx = (int)floorf((x - h.x0) * h.inv_w), cy = (int)floorf((y - h.y0) * h.inv_w);
    if (cx < 0 || cy < 0 || cx >= (int)h.cols_x || cy >= (int)h.cols_y) return -1;
    return cy * (int)h.cols_x + cx;
}

__global__ void height_accumulate(const HeightArgs h)
{
    const uint32_t nv = (uint32_t)min(*h.totals, (unsigned long long)h.vert_capacity);
    const uint32_t cols = h.cols_x * h.cols_y;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const uww_vert_color q = h.verts[v];
        const int c = column_of(h, q.pos[0], q.pos[1]);
        if (c < 0) continue;
        atomicAdd(reinterpret_cast<unsigned long long*>(h.sum_z + c),
                  (unsigned long long)__double2ll_rn((double)q.pos[2] * kHeightFix));
        atomicAdd(h.count + c, 1ull);
    }
    (void)cols;
}

__global__ void height_grad(const HeightArgs h)
{
    const uint32_t nv = (uint32_t)min(*h.totals, (unsigned long long)h.vert_capacity);
    const uint32_t cols = h.cols_x * h.cols_y;
    const float inv_cols = 1.f / (float)cols;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
        const uww_vert_color q = h.verts[i];
        const int c = column_of(h, q.pos[0], q.pos[1]);
        float gz = 0.f;
        if (c >= 0) {
            const float cnt = (float)h.count[c];
            gz = 2.f * (column_mean(h, c) - h.target[c]) / cnt * inv_cols;
        }
        h.pos_grad[3 * (size_t)i] = 0.f;
        h.pos_grad[3 * (size_t)i + 1] = 0.f;
        h.pos_grad[3 * (size_t)i + 2] = gz;
    }
}

// The loss, by one CTA of 1024 threads in a fixed order: per thread a strided
// sum over the columns, then a tree over the threads.
__global__ void __launch_bounds__(1024) height_loss_reduce(const HeightArgs h)
{
    __shared__ float part[1024];
    const uint32_t cols = h.cols_x * h.cols_y;
    const float inv_cols = 1.f / (float)cols;
    float s = 0.f;
    for (uint32_t c = threadIdx.x; c < cols; c += blockDim.x)
        if (h.count[c]) {
            const float r = column_mean(h, (int)c) - h.target[c];
            s += r * r * inv_cols;
        }
    part[threadIdx.x] = s;
    __syncthreads();
    for (unsigned o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *h.loss = part[0];
}

template <class O, int KMAX>
cudaError_t launch_backward_t(const DevParams& p, const AdjointArgs& a, int grid, cudaStream_t s)
{
    backward_kernel<O, KMAX><<<grid, kBwdThreads, 0, s>>>(p, a);
    return cudaGetLastError();
}

// CTAs of the backward: every resident one (the assignment of vertices to
// threads depends only on this number)
template <class O, int KMAX>
int backward_grid_t(int sms)
{
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, backward_kernel<O, KMAX>, kBwdThreads, 0) != cudaSuccess ||
        occ < 1) {
        cudaGetLastError();
        occ = 1;
    }
    return occ * sms;
}

template <class O>
int backward_grid_o(const DevParams& p, int sms)
{
    if (p.octaves <= 4) return backward_grid_t<O, 4>(sms);
    if (p.octaves <= 8) return backward_grid_t<O, 8>(sms);
    return backward_grid_t<O, 16>(sms);
}

template <class O>
cudaError_t launch_backward_o(const DevParams& p, const AdjointArgs& a, int grid, cudaStream_t s)
{
    if (p.octaves <= 4) return launch_backward_t<O, 4>(p, a, grid, s);
    if (p.octaves <= 8) return launch_backward_t<O, 8>(p, a, grid, s);
    return launch_backward_t<O, 16>(p, a, grid, s);
}

int kmax_for(int octaves) { return octaves <= 4 ? 4 : octaves <= 8 ? 8 : 16; }

}  // namespace
}  // namespace uww

using namespace uww;

#pragma GCC visibility push(default)
extern "C" {

int uww_forward(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                const uww_mesh_out* out, uint32_t* d_edge_ids)
{
    if (!ctx || !d_edge_ids) return UWW_ERR_INVALID_ARG;
    int st = check_mesh_out(out);
    if (st) return st;
    if (max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    if (n == 0) {
        if (out->totals)
            return status_from_cuda(cudaMemsetAsync(out->totals, 0, 4 * sizeof(uint64_t), ctx->stream), "cudaMemsetAsync");
        return UWW_OK;
    }
    if (!d_chunks) return UWW_ERR_INVALID_ARG;
    return launch_batched(ctx, d_chunks, n, max_cells, out, d_edge_ids, nullptr);
}

int uww_backward(uww_ctx* ctx, const uww_chunk_desc* d_chunks, uint32_t n, uint32_t max_cells,
                 const uww_chunk_record* d_records, const uint32_t* d_edge_ids, const float* d_pos_grad,
                 float* d_theta_grad, float* d_sample_grad, uint64_t sample_capacity)
{
    if (!ctx || !d_theta_grad) return UWW_ERR_INVALID_ARG;
    if (max_cells < 1 || max_cells > UWW_MAX_CELLS) return UWW_ERR_INVALID_ARG;
    cudaStream_t s = ctx->stream;
    if (d_sample_grad && sample_capacity) {
        int st = status_from_cuda(cudaMemsetAsync(d_sample_grad, 0, sample_capacity * sizeof(float), s), "cudaMemsetAsync");
        if (st) return st;
    }
    const int K = ctx->dev.octaves;
    if (n == 0)
        return status_from_cuda(cudaMemsetAsync(d_theta_grad, 0, (size_t)(K + 5) * sizeof(float), s), "cudaMemsetAsync");
    if (!d_chunks || !d_records || !d_edge_ids || !d_pos_grad) return UWW_ERR_INVALID_ARG;
    const int NV = kmax_for(K) + 5;
    const bool exact = ctx->dev.math_mode == UWW_MATH_EXACT;
    const int grid = exact ? backward_grid_o<ExactOps>(ctx->dev, ctx->num_sms) : backward_grid_o<FastOps>(ctx->dev, ctx->num_sms);
    int st = ensure_device_of(&ctx->d_adj_part, &ctx->adj_part_cap, (size_t)grid * NV * sizeof(float));
    if (st) return st;
    if (!ctx->d_adj_counter) {
        cudaError_t e = cudaMalloc((void**)&ctx->d_adj_counter, sizeof(unsigned int));
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_adj_counter, 0, sizeof(unsigned int), s);
        if (e != cudaSuccess) {
            cudaFree(ctx->d_adj_counter);
            ctx->d_adj_counter = nullptr;
            return status_from_cuda(e, "cudaMalloc");
        }
    }
    AdjointArgs a;
    std::memset(&a, 0, sizeof(a));
    a.chunks = d_chunks;
    a.records = d_records;
    a.edge_ids = d_edge_ids;
    a.pos_grad = d_pos_grad;
    a.sample_grad = d_sample_grad;
    a.sample_capacity = d_sample_grad ? sample_capacity : 0;
    a.part = ctx->d_adj_part;
    a.counter = ctx->d_adj_counter;
    a.theta_grad = d_theta_grad;
    a.n = n;
    a.max_cells = max_cells;
    const cudaError_t e = exact ? launch_backward_o<ExactOps>(ctx->dev, a, grid, s)
                                : launch_backward_o<FastOps>(ctx->dev, a, grid, s);
    return status_from_cuda(e, "backward kernel launch");
}

int uww_height_loss(uww_ctx* ctx, const uww_vert_color* d_verts, const uint64_t* d_totals, uint32_t vert_capacity,
                    float x0, float y0, float column, uint32_t cols_x, uint32_t cols_y, const float* d_target,
                    float* d_work, float* d_pos_grad, float* d_loss)
{
    if (!ctx || !d_verts || !d_totals || !d_target || !d_work || !d_pos_grad || !d_loss) return UWW_ERR_INVALID_ARG;
    if (!(column > 0.f) || cols_x == 0 || cols_y == 0) return UWW_ERR_INVALID_ARG;
    if (!aligned_to(d_work, 8)) return UWW_ERR_INVALID_ARG;
    cudaStream_t s = ctx->stream;
    const size_t cols = (size_t)cols_x * cols_y;
    cudaError_t e = cudaMemsetAsync(d_work, 0, 4 * cols * sizeof(float), s);
    if (e != cudaSuccess) return status_from_cuda(e, "cudaMemsetAsync");
    HeightArgs h;
    h.verts = d_verts;
    h.totals = reinterpret_cast<const unsigned long long*>(d_totals);
    h.vert_capacity = vert_capacity;
    h.x0 = x0;
    h.y0 = y0;
    h.inv_w = 1.f / column;
    h.cols_x = cols_x;
    h.cols_y = cols_y;
    h.target = d_target;
    h.sum_z = reinterpret_cast<long long*>(d_work);
    h.count = reinterpret_cast<unsigned long long*>(d_work) + cols;
    h.pos_grad = d_pos_grad;
    h.loss = d_loss;
    const int grid = std::max(1, std::min<int>(ctx->num_sms * 8, (int)((std::max<size_t>(vert_capacity, cols) + 255) / 256)));
    height_accumulate<<<grid, 256, 0, s>>>(h);
    height_grad<<<grid, 256, 0, s>>>(h);
    height_loss_reduce<<<1, 1024, 0, s>>>(h);
    return status_from_cuda(cudaGetLastError(), "height loss kernel launch");
}

}  // extern "C"
#pragma GCC visibility pop
