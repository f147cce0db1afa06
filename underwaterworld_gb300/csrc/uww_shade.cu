// uww_shade.cu -- the terrain shader's arithmetic as a CUDA pass over a
// build's vertices, into headless buffers (no graphics API on this path):
// terrain.wgsl vs_main (clip position, distance to the sub, the sub's
// spotlight term) and fs_main (distance fog) evaluated at each vertex.
// Reference: underwater_world/src/terrain.wgsl:26-59, CameraUniform of
// camera.rs:69-79.  WGSL built-ins restated: length = sqrt(dot),
// smoothstep(a, b, x) = t^2 (3 - 2t) with t = clamp((x - a) / (b - a), 0, 1),
// mix(a, b, t) = a (1 - t) + b t.  acos/cos are the CUDA library functions.
#include <cuda_runtime.h>

#include <algorithm>

#include "uww_internal.h"

namespace uww {
namespace {

__device__ __forceinline__ float smoothstep_w(float a, float b, float x)
{
    const float t = fminf(fmaxf(__fdiv_rn(__fsub_rn(x, a), __fsub_rn(b, a)), 0.f), 1.f);
    return __fmul_rn(__fmul_rn(t, t), __fsub_rn(3.f, __fmul_rn(2.f, t)));
}

__device__ __forceinline__ float dot3(const float* a, const float* b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])), __fmul_rn(a[2], b[2]));
}

__global__ void shade_kernel(const uww_camera_uniform cam, const uww_vert_color* __restrict__ verts,
                             const unsigned long long* __restrict__ totals, uint32_t count, uint32_t capacity,
                             float* __restrict__ clip, float* __restrict__ rgb, float* __restrict__ dist_light)
{
    const uint32_t nv = totals ? (uint32_t)min(*totals, (unsigned long long)capacity) : min(count, capacity);
    const float half_pi = __fdiv_rn(3.14159f, 2.f);
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const uww_vert_color vc = verts[v];
        const float* p = vc.pos;
        if (clip) {
            // view_proj * vec4(position, 1), column-major
#pragma unroll
            for (int i = 0; i < 4; ++i)
                clip[4 * (size_t)v + i] =
                    __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(cam.view_proj[i], p[0]), __fmul_rn(cam.view_proj[4 + i], p[1])),
                                        __fmul_rn(cam.view_proj[8 + i], p[2])),
                              cam.view_proj[12 + i]);
        }
        const float dv[3] = {__fsub_rn(p[0], cam.sub_pos[0]), __fsub_rn(p[1], cam.sub_pos[1]), __fsub_rn(p[2], cam.sub_pos[2])};
        const float dist = __fsqrt_rn(dot3(dv, dv));
        const float cos_angle = __fdiv_rn(dot3(dv, cam.sub_forward), __fmul_rn(dist, __fsqrt_rn(dot3(cam.sub_forward, cam.sub_forward))));
        const float angle = acosf(cos_angle);
        const float light0 = __fmul_rn(cosf(__fmul_rn(angle, 3.f)), angle < half_pi ? 1.f : 0.f);
        const float light = smoothstep_w(0.f, 1.f, light0);
        // fs_main at the vertex
        const float min_dist_value = smoothstep_w(0.f, 20.f, fminf(fmaxf(dist, 0.f), 20.f));
        const float max_dist_value = smoothstep_w(0.f, 45.f, fminf(fmaxf(dist, 0.f), 45.f));
        const float dark = fminf(fmaxf(__fsub_rn(1.f, light), max_dist_value), min_dist_value);
        if (rgb) {
#pragma unroll
            for (int i = 0; i < 3; ++i)
                rgb[3 * (size_t)v + i] = __fadd_rn(__fmul_rn(vc.color[i], __fsub_rn(1.f, dark)), __fmul_rn(cam.fog_color[i], dark));
        }
        if (dist_light) {
            dist_light[2 * (size_t)v] = dist;
            dist_light[2 * (size_t)v + 1] = light;
        }
    }
}

}  // namespace
}  // namespace uww

using namespace uww;

#pragma GCC visibility push(default)
extern "C" int uww_shade_vertices(uww_ctx* ctx, const uww_camera_uniform* cam, const uww_vert_color* d_verts,
                                  const uint64_t* d_totals, uint32_t count, uint32_t vert_capacity, float* d_clip,
                                  float* d_rgb, float* d_dist_light)
{
    if (!ctx || !cam || !d_verts) return UWW_ERR_INVALID_ARG;
    if (!d_clip && !d_rgb && !d_dist_light) return UWW_OK;
    const uint32_t work = d_totals ? vert_capacity : std::min(count, vert_capacity);
    if (work == 0) return UWW_OK;
    const int grid = (int)std::min<uint32_t>((work + 255) / 256, (uint32_t)ctx->num_sms * 8);
    shade_kernel<<<grid, 256, 0, ctx->stream>>>(*cam, d_verts, reinterpret_cast<const unsigned long long*>(d_totals),
                                                count, vert_capacity, d_clip, d_rgb, d_dist_light);
    return status_from_cuda(cudaGetLastError(), "shade kernel launch");
}
#pragma GCC visibility pop
