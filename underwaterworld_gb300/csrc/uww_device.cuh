// uww_device.cuh -- device-side density: seeded Perlin, fBm, depth bias,
// analytic gradient, and the per-vertex colour ramp.
//
// Two arithmetic policies:
//   ExactOps -- every add/sub/mul is a separately rounded IEEE op
//               (__fadd_rn/__fsub_rn/__fmul_rn are never contracted to FMA),
//               in the reference's operation order.  This is the parity build.
//   FastOps  -- plain operators; nvcc contracts them to FMA (fast build).
// sqrt, floor and fmod are IEEE-exact in both; division is IEEE in the parity
// build and the hardware approximate quotient (O::div) in the fast build's
// edge interpolation.
//
// Reference: perlin_util.rs:6-29 (fBm + terraced bias), the noise 0.8.2
// crate's perlin_3d behind noise::Perlin::get (perlin_util.rs:13), and the
// colour path of chunk.rs:208-219 with util.rs:93-153.
#pragma once
#include <stdint.h>

#include <type_traits>

#include "uww.h"

namespace uww {

// Kernel-argument block: everything a launch needs, passed by value so that a
// captured CUDA graph carries its own copy (no device allocation for tables).
struct DevParams {
    uint8_t perm[256];                 // noise::Perlin::new(seed) permutation
    float mult[UWW_MAX_OCTAVES];       // frequency multiplier per octave (1, lac, lac^2, ...)
    float amp[UWW_MAX_OCTAVES];        // amplitude per octave
    int32_t octaves;
    int32_t chunk_size;
    float base_freq;
    float iso_level;
    float offset[3];
    int32_t normalize;
    int32_t bias_mode;
    float bias_a, bias_b, bias_c;
    float color_min_z, color_max_z;
    uint32_t outputs;
    int32_t dedup_mode;
    int32_t math_mode;
};

struct ExactOps {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};

struct FastOps {
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    // the hardware reciprocal-based quotient (about 2 ulp), for |b| < 2^126
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
};

// Gradient table of the noise crate: 16 entries over the 12 cube-edge
// directions, value = (+-u) + (+-v).  Nibble h of this word encodes entry h:
// bit0 u is y (else x), bit1 negate u, bit2 v is z (else y), bit3 negate v.
constexpr unsigned long long kGradCode = 0xF720FD75EC64A820ull;

template <class O>
__device__ __forceinline__ float grad_dot(int h, float x, float y, float z)
{
    const unsigned c = (unsigned)(kGradCode >> ((h & 15) * 4)) & 15u;
    float u = (c & 1u) ? y : x;
    float v = (c & 4u) ? z : y;
    u = (c & 2u) ? -u : u;
    v = (c & 8u) ? -v : v;
    return O::add(u, v);
}

// gradient vector of entry h, components in {-1, 0, 1}
__device__ __forceinline__ void grad_vec(int h, float& gx, float& gy, float& gz)
{
    const unsigned c = (unsigned)(kGradCode >> ((h & 15) * 4)) & 15u;
    const float su = (c & 2u) ? -1.f : 1.f, sv = (c & 8u) ? -1.f : 1.f;
    gx = (c & 1u) ? 0.f : su;
    gy = ((c & 1u) ? su : 0.f) + ((c & 4u) ? 0.f : sv);
    gz = (c & 4u) ? sv : 0.f;
}

__device__ __forceinline__ int hash3(const uint8_t* P, int x, int y, int z)
{
    return P[P[P[x & 255] ^ (y & 255)] ^ (z & 255)];
}

template <class O>
__device__ __forceinline__ float fade(float t)
{   // t*t*t*(t*(t*6-15)+10)
    return O::mul(O::mul(O::mul(t, t), t), O::add(O::mul(t, O::sub(O::mul(t, 6.f), 15.f)), 10.f));
}

template <class O>
__device__ __forceinline__ float dfade(float t)
{   // 30*t*t*(t*(t-2)+1)
    return O::mul(O::mul(O::mul(30.f, t), t), O::add(O::mul(t, O::sub(t, 2.f)), 1.f));
}

// k0 + k1 a + k2 b + k3 c + k4 a b + k5 a c + k6 b c + k7 a b c, left to right
template <class O>
__device__ __forceinline__ float kpoly(float k0, float k1, float k2, float k3, float k4, float k5, float k6,
                                       float k7, float a, float b, float c)
{
    float r = O::add(k0, O::mul(k1, a));
    r = O::add(r, O::mul(k2, b));
    r = O::add(r, O::mul(k3, c));
    r = O::add(r, O::mul(O::mul(k4, a), b));
    r = O::add(r, O::mul(O::mul(k5, a), c));
    r = O::add(r, O::mul(O::mul(k6, b), c));
    r = O::add(r, O::mul(O::mul(O::mul(k7, a), b), c));
    return r;
}

constexpr float kPerlinScale = 1.1547005383792515f;  // 2/sqrt(3)

// One Perlin evaluation in the crate's formulation.  If GRAD, g receives
// d(value)/d(p).
template <class O, bool GRAD>
__device__ __forceinline__ float perlin(const uint8_t* P, float px, float py, float pz, float* g)
{
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    const float dx = O::sub(px, fx), dy = O::sub(py, fy), dz = O::sub(pz, fz);
    const float dx1 = O::sub(dx, 1.f), dy1 = O::sub(dy, 1.f), dz1 = O::sub(dz, 1.f);

    const int a0 = P[ix & 255], a1 = P[(ix + 1) & 255];
    const int b00 = P[a0 ^ (iy & 255)], b01 = P[a0 ^ ((iy + 1) & 255)];
    const int b10 = P[a1 ^ (iy & 255)], b11 = P[a1 ^ ((iy + 1) & 255)];
    const int z0 = iz & 255, z1 = (iz + 1) & 255;
    const int h000 = P[b00 ^ z0], h001 = P[b00 ^ z1];
    const int h010 = P[b01 ^ z0], h011 = P[b01 ^ z1];
    const int h100 = P[b10 ^ z0], h101 = P[b10 ^ z1];
    const int h110 = P[b11 ^ z0], h111 = P[b11 ^ z1];

    const float g000 = grad_dot<O>(h000, dx, dy, dz);
    const float g100 = grad_dot<O>(h100, dx1, dy, dz);
    const float g010 = grad_dot<O>(h010, dx, dy1, dz);
    const float g110 = grad_dot<O>(h110, dx1, dy1, dz);
    const float g001 = grad_dot<O>(h001, dx, dy, dz1);
    const float g101 = grad_dot<O>(h101, dx1, dy, dz1);
    const float g011 = grad_dot<O>(h011, dx, dy1, dz1);
    const float g111 = grad_dot<O>(h111, dx1, dy1, dz1);

    const float a = fade<O>(dx), b = fade<O>(dy), c = fade<O>(dz);

    const float k0 = g000;
    const float k1 = O::sub(g100, g000);
    const float k2 = O::sub(g010, g000);
    const float k3 = O::sub(g001, g000);
    const float k4 = O::sub(O::sub(O::add(g000, g110), g100), g010);
    const float k5 = O::sub(O::sub(O::add(g000, g101), g100), g001);
    const float k6 = O::sub(O::sub(O::add(g000, g011), g010), g001);
    const float k7 = O::sub(O::sub(O::sub(O::sub(O::add(O::add(O::add(g100, g010), g001), g111), g000), g110), g101), g011);

    if (GRAD) {
        float G[8][3];
        grad_vec(h000, G[0][0], G[0][1], G[0][2]);
        grad_vec(h100, G[1][0], G[1][1], G[1][2]);
        grad_vec(h010, G[2][0], G[2][1], G[2][2]);
        grad_vec(h110, G[3][0], G[3][1], G[3][2]);
        grad_vec(h001, G[4][0], G[4][1], G[4][2]);
        grad_vec(h101, G[5][0], G[5][1], G[5][2]);
        grad_vec(h011, G[6][0], G[6][1], G[6][2]);
        grad_vec(h111, G[7][0], G[7][1], G[7][2]);
        const float da = dfade<O>(dx), db = dfade<O>(dy), dc = dfade<O>(dz);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            // the j's are small integers: exact in any order
            const float q000 = G[0][ax], q100 = G[1][ax], q010 = G[2][ax], q110 = G[3][ax];
            const float q001 = G[4][ax], q101 = G[5][ax], q011 = G[6][ax], q111 = G[7][ax];
            const float j0 = q000, j1 = q100 - q000, j2 = q010 - q000, j3 = q001 - q000;
            const float j4 = q000 + q110 - q100 - q010;
            const float j5 = q000 + q101 - q100 - q001;
            const float j6 = q000 + q011 - q010 - q001;
            const float j7 = q100 + q010 + q001 + q111 - q000 - q110 - q101 - q011;
            float s = kpoly<O>(j0, j1, j2, j3, j4, j5, j6, j7, a, b, c);
            float t;
            if (ax == 0) t = O::mul(da, O::add(O::add(O::add(k1, O::mul(k4, b)), O::mul(k5, c)), O::mul(O::mul(k7, b), c)));
            else if (ax == 1) t = O::mul(db, O::add(O::add(O::add(k2, O::mul(k4, a)), O::mul(k6, c)), O::mul(O::mul(k7, a), c)));
            else t = O::mul(dc, O::add(O::add(O::add(k3, O::mul(k5, a)), O::mul(k6, b)), O::mul(O::mul(k7, a), b)));
            s = O::add(s, t);
            g[ax] = O::mul(s, kPerlinScale);
        }
    }
    return O::mul(kpoly<O>(k0, k1, k2, k3, k4, k5, k6, k7, a, b, c), kPerlinScale);
}

// perlin_3d_octaves (perlin_util.rs:6-22) at noise-space point n.
template <class O, bool GRAD>
__device__ __forceinline__ float fbm(const DevParams& p, const uint8_t* P, float nx, float ny, float nz, float* g)
{
    float total = 0.f, maxv = 0.f;
    float gt0 = 0.f, gt1 = 0.f, gt2 = 0.f;
    // unrolled so that independent octaves overlap their table-lookup chains
#pragma unroll 4
    for (int k = 0; k < p.octaves; ++k) {
        const float m = p.mult[k], am = p.amp[k];
        float gk[3];
        const float v = perlin<O, GRAD>(P, O::mul(nx, m), O::mul(ny, m), O::mul(nz, m), gk);
        total = O::add(total, O::mul(v, am));
        maxv = O::add(maxv, am);
        if (GRAD) {
            gt0 = O::add(gt0, O::mul(O::mul(gk[0], am), m));
            gt1 = O::add(gt1, O::mul(O::mul(gk[1], am), m));
            gt2 = O::add(gt2, O::mul(O::mul(gk[2], am), m));
        }
    }
    if (p.normalize) {
        if (GRAD) { g[0] = __fdiv_rn(gt0, maxv); g[1] = __fdiv_rn(gt1, maxv); g[2] = __fdiv_rn(gt2, maxv); }
        return __fdiv_rn(total, maxv);
    }
    if (GRAD) { g[0] = gt0; g[1] = gt1; g[2] = gt2; }
    return total;
}

// iso_at (perlin_util.rs:24-29), generalised by bias_mode, at a world point.
template <class O, bool GRAD>
__device__ __forceinline__ float density(const DevParams& p, const uint8_t* P, float wx, float wy, float wz, float* g)
{
    const float nx = O::mul(O::add(wx, p.offset[0]), p.base_freq);
    const float ny = O::mul(O::add(wy, p.offset[1]), p.base_freq);
    const float nz = O::mul(O::add(wz, p.offset[2]), p.base_freq);
    float gn[3];
    const float f = fbm<O, GRAD>(p, P, nx, ny, nz, gn);
    if (GRAD) {
        g[0] = O::mul(gn[0], p.base_freq);
        g[1] = O::mul(gn[1], p.base_freq);
        g[2] = O::mul(gn[2], p.base_freq);
    }
    if (p.bias_mode == UWW_BIAS_TERRACED) {
        const float adj = __fdiv_rn(O::mul(nz, p.bias_a), p.bias_b);
        return O::sub(O::add(adj, f), fmodf(adj, p.bias_c));
    }
    if (p.bias_mode == UWW_BIAS_LINEAR) {
        if (GRAD) g[2] = O::add(g[2], p.bias_a);
        return O::add(f, O::mul(p.bias_a, O::sub(wz, p.bias_b)));
    }
    return f;
}

// Fast build: density gradient at a world point for vertex normals.  Same
// Perlin/fBm maths, written as trilinear interpolation with FMA, the corner
// gradient vectors read from gp (gradient of P[i], the last hash lookup):
//   n      = sum_c w_c v_c,          v_c = g_c . (d - o_c),
//   dn/dd  = sum_c w_c g_c + (da (Y1 - Y0), db (.), dc (.)),
// where Y1 - Y0 is the difference of the two faces' bilinear interpolants.
__device__ __forceinline__ void density_grad_fast(const DevParams& p, const uint8_t* P, const float4* gp, float wx,
                                                  float wy, float wz, float g[3])
{
    const float bf = p.base_freq;
    const float nx = (wx + p.offset[0]) * bf, ny = (wy + p.offset[1]) * bf, nz = (wz + p.offset[2]) * bf;
    float gx = 0.f, gy = 0.f, gz = 0.f, msum = 0.f;
    // unrolled so that independent octaves overlap their table-lookup chains
#pragma unroll 4
    for (int k = 0; k < p.octaves; ++k) {
        const float m = p.mult[k], am = p.amp[k];
        msum += am;
        const float qx = nx * m, qy = ny * m, qz = nz * m;
        const float fx = floorf(qx), fy = floorf(qy), fz = floorf(qz);
        const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
        const float dx = qx - fx, dy = qy - fy, dz = qz - fz;
        const float dx1 = dx - 1.f, dy1 = dy - 1.f, dz1 = dz - 1.f;
        const int a0 = P[ix & 255], a1 = P[(ix + 1) & 255];
        const int b00 = P[a0 ^ (iy & 255)], b01 = P[a0 ^ ((iy + 1) & 255)];
        const int b10 = P[a1 ^ (iy & 255)], b11 = P[a1 ^ ((iy + 1) & 255)];
        const int z0 = iz & 255, z1 = (iz + 1) & 255;
        // corner index bits: x 4, y 2, z 1
        const float4 c0 = gp[b00 ^ z0], c1 = gp[b00 ^ z1], c2 = gp[b01 ^ z0], c3 = gp[b01 ^ z1];
        const float4 c4 = gp[b10 ^ z0], c5 = gp[b10 ^ z1], c6 = gp[b11 ^ z0], c7 = gp[b11 ^ z1];
        const float v0 = fmaf(c0.x, dx, fmaf(c0.y, dy, c0.z * dz));
        const float v1 = fmaf(c1.x, dx, fmaf(c1.y, dy, c1.z * dz1));
        const float v2 = fmaf(c2.x, dx, fmaf(c2.y, dy1, c2.z * dz));
        const float v3 = fmaf(c3.x, dx, fmaf(c3.y, dy1, c3.z * dz1));
        const float v4 = fmaf(c4.x, dx1, fmaf(c4.y, dy, c4.z * dz));
        const float v5 = fmaf(c5.x, dx1, fmaf(c5.y, dy, c5.z * dz1));
        const float v6 = fmaf(c6.x, dx1, fmaf(c6.y, dy1, c6.z * dz));
        const float v7 = fmaf(c7.x, dx1, fmaf(c7.y, dy1, c7.z * dz1));
        const float a = fade<FastOps>(dx), b = fade<FastOps>(dy), c = fade<FastOps>(dz);
        const float da = dfade<FastOps>(dx), db = dfade<FastOps>(dy), dc = dfade<FastOps>(dz);
        // trilinear weights as lerps: along z, then y, then x
        auto lerp = [](float t, float u, float v) { return fmaf(t, v - u, u); };
        const float z00 = lerp(c, v0, v1), z01 = lerp(c, v2, v3), z10 = lerp(c, v4, v5), z11 = lerp(c, v6, v7);
        const float y0 = lerp(b, z00, z01), y1 = lerp(b, z10, z11);
        // d/dx: da * (face x1 - face x0)
        float tx = da * (y1 - y0);
        // d/dy: db * lerp_x(z_y1 - z_y0)
        float ty = db * lerp(a, z01 - z00, z11 - z10);
        // d/dz: dc * lerp_x(lerp_y(v_z1 - v_z0))
        float tz = dc * lerp(a, lerp(b, v1 - v0, v3 - v2), lerp(b, v5 - v4, v7 - v6));
        // + sum_c w_c g_c, as trilinear interpolation of each component
        auto tri = [&](float e0, float e1, float e2, float e3, float e4, float e5, float e6, float e7) {
            return lerp(a, lerp(b, lerp(c, e0, e1), lerp(c, e2, e3)), lerp(b, lerp(c, e4, e5), lerp(c, e6, e7)));
        };
        tx += tri(c0.x, c1.x, c2.x, c3.x, c4.x, c5.x, c6.x, c7.x);
        ty += tri(c0.y, c1.y, c2.y, c3.y, c4.y, c5.y, c6.y, c7.y);
        tz += tri(c0.z, c1.z, c2.z, c3.z, c4.z, c5.z, c6.z, c7.z);
        const float s = am * m;
        gx = fmaf(tx, s, gx);
        gy = fmaf(ty, s, gy);
        gz = fmaf(tz, s, gz);
    }
    float scale = kPerlinScale * bf;
    if (p.normalize) scale = scale / msum;
    g[0] = gx * scale;
    g[1] = gy * scale;
    g[2] = gz * scale;
    if (p.bias_mode == UWW_BIAS_LINEAR) g[2] += p.bias_a;
}

// Unit normal from the density gradient (util.rs:61-64 safe_normalize).
template <class O>
__device__ __forceinline__ void safe_normalize(float g[3])
{
    if constexpr (std::is_same<O, FastOps>::value) {
        // fast build: one reciprocal square root instead of a square root and three divisions
        const float d = fmaf(g[0], g[0], fmaf(g[1], g[1], g[2] * g[2]));
        if (d != 0.f) {
            const float r = rsqrtf(d);
            g[0] *= r;
            g[1] *= r;
            g[2] *= r;
        }
        return;
    }
    const float mag = __fsqrt_rn(O::add(O::add(O::mul(g[0], g[0]), O::mul(g[1], g[1])), O::mul(g[2], g[2])));
    if (mag != 0.f) {
        g[0] = __fdiv_rn(g[0], mag);
        g[1] = __fdiv_rn(g[1], mag);
        g[2] = __fdiv_rn(g[2], mag);
    }
}

// Per-vertex colour: chunk.rs:208-219 -> util.rs:93-95, 122-153, 106-112.
// fmodf(x, y) for y > 0, bit for bit: x itself when |x| < y, and x - y or
// x - 2y when x lies in [y, 3y) -- fmod's result is exact, and so are these
// differences (Sterbenz's lemma) -- else fmodf.  The colour ramp's arguments
// stay in those ranges, where fmodf's general path is the slow part.
__device__ __forceinline__ float fmod_pos(float x, float y)
{
    if (fabsf(x) < y) return x;
    if (x >= y && x < 2.0f * y) return __fsub_rn(x, y);
    if (x >= 2.0f * y && x < 3.0f * y) return __fsub_rn(x, 2.0f * y);
    return fmodf(x, y);
}

template <class O>
__device__ __forceinline__ void vertex_color(const DevParams& p, float world_z, int corner_b, float out[3])
{
    // divisions: IEEE in the parity build, the approximate quotient in the fast build
    const float ratio = O::div(world_z, (float)p.chunk_size);
    const float mix = O::div(O::sub(ratio, p.color_min_z), O::sub(p.color_max_z, p.color_min_z));
    const float vi = O::div((float)(corner_b % 3), 9.0f);
    const float hue0 = O::add(-150.0f, O::mul(210.0f, mix));  // MIN_HUE + (MAX_HUE - MIN_HUE) * mix
    const float value = O::add(0.4f, vi);                      // BASE_VALUE + value_intensity
    const float r0 = fmod_pos(hue0, 360.0f);
    const float hue = r0 < 0.f ? O::add(r0, 360.0f) : r0;      // rem_euclid
    const float c = O::mul(value, 0.6f);                       // SATURATION
    const float h = O::div(hue, 60.0f);
    const float x = O::mul(c, O::sub(1.0f, fabsf(O::sub(fmod_pos(h, 2.0f), 1.0f))));
    const float m = O::sub(value, c);
    float r, gg, b;
    if (0.f <= h && h < 1.f)      { r = c; gg = x; b = 0.f; }
    else if (1.f <= h && h < 2.f) { r = x; gg = c; b = 0.f; }
    else if (2.f <= h && h < 3.f) { r = 0.f; gg = c; b = x; }
    else if (3.f <= h && h < 4.f) { r = 0.f; gg = x; b = c; }
    else if (4.f <= h && h < 5.f) { r = x; gg = 0.f; b = c; }
    else                          { r = c; gg = 0.f; b = x; }
    const float rgb[3] = {O::mul(O::add(r, m), 255.0f), O::mul(O::add(gg, m), 255.0f), O::mul(O::add(b, m), 255.0f)};
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        const float base = O::div(O::add(O::div(rgb[i], 255.0f), 0.055f), 1.055f);
        // parity build: powf; fast build: the hardware exp2/log2 pair (base > 0)
        out[i] = std::is_same<O, FastOps>::value ? __powf(base, 2.4f) : powf(base, 2.4f);
    }
}

}  // namespace uww
