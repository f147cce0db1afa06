"""terrain.wgsl (terrain.wgsl:26-59) evaluated per vertex on the GPU against
the CPU restatement.  Clip positions and distances are exact (same f32
operation order); the spotlight and fog use acos/cos, whose last-bit
rounding differs between CUDA and libm: 2e-5 absolute on values in [0, 1]."""
import ctypes as C

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import DeviceArray
from underwaterworld_gb300.schedule import frustum_matrix

pytestmark = pytest.mark.gpu


def camera(sub, forward, fog=(0.0, 0.12, 0.2)):
    cam = abi.CameraUniform()
    eye = np.asarray(sub, np.float32) - 5 * np.asarray(forward, np.float32)
    for i, v in enumerate(frustum_matrix(eye, np.asarray(sub, np.float32), (0, 0, 1), 45.0, 16 / 9)):
        cam.view_proj[i] = float(v)
    for i in range(3):
        cam.fog_color[i], cam.sub_pos[i], cam.sub_forward[i] = fog[i], float(sub[i]), float(forward[i])
    return cam


def test_shading_matches_the_oracle(ctx_factory, oracle):
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_COLOR)
    ctx = ctx_factory(p)
    vcap = 1 << 20
    d_desc = ctx.upload(d)
    d_v, d_i, d_r, d_t = DeviceArray(vcap * 24), DeviceArray(4 << 22), DeviceArray(len(d) * 32), DeviceArray(32)
    out = abi.MeshOut(d_v.ptr, None, d_i.ptr, None, None, d_r.ptr, d_t.ptr, vcap, 1 << 22, 0, 0)
    abi.check(abi.lib().uww_build_chunks(ctx.h, C.c_void_p(d_desc.ptr), len(d), 12, C.byref(out)))
    ctx.sync()
    nv = int(ctx.download(d_t, (4,), np.uint64)[0])
    verts = ctx.download(d_v, (nv,), abi.VERT_COLOR_DTYPE)
    d_clip, d_rgb, d_dl = DeviceArray(vcap * 16), DeviceArray(vcap * 12), DeviceArray(vcap * 8)
    for sub, fwd in [((3.0, -2.0, 1.0), (1.0, 0.2, -0.1)), ((-20.0, 10.0, -5.0), (0.0, -1.0, 0.3))]:
        cam = camera(sub, fwd)
        # the vertex count straight from the build's totals
        abi.check(abi.lib().uww_shade_vertices(ctx.h, C.byref(cam), C.c_void_p(d_v.ptr), C.c_void_p(d_t.ptr), 0, vcap,
                                               C.c_void_p(d_clip.ptr), C.c_void_p(d_rgb.ptr), C.c_void_p(d_dl.ptr)))
        ctx.sync()
        clip = ctx.download(d_clip, (nv, 4), np.float32)
        rgb = ctx.download(d_rgb, (nv, 3), np.float32)
        dl = ctx.download(d_dl, (nv, 2), np.float32)
        w_clip, w_rgb, w_dl = oracle.shade_vertices(cam, verts)
        np.testing.assert_array_equal(clip, w_clip)
        np.testing.assert_array_equal(dl[:, 0], w_dl[:, 0])
        np.testing.assert_allclose(dl[:, 1], w_dl[:, 1], rtol=0, atol=2e-5)
        np.testing.assert_allclose(rgb, w_rgb, rtol=0, atol=2e-5)
        assert (dl[:, 1] > 0).any() and (dl[:, 1] == 0).any()
