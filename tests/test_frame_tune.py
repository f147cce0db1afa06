"""Per-frame build captured in a CUDA graph (uww_frame_*) and the autotuner
(uww_autotune): both must give exactly the output of a plain uww_build_chunks
call on the same descriptors."""
import ctypes as C

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import DeviceArray, make_descs
from underwaterworld_gb300.frame import FrameBuilder, autotune

pytestmark = pytest.mark.gpu

OUT = abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS


def direct_build(ctx, descs, vcap, icap):
    b = ctx.build_chunks_device(descs, vcap, icap)
    assert b.status == abi.UWW_OK
    return b


def test_frame_graph_matches_direct_builds(ctx_factory):
    p, d = workloads.uniform_grid(seed=2, outputs=OUT)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    vcap, icap = 1 << 20, 1 << 22
    fb = FrameBuilder(ctx, len(d), 12, vcap, icap)
    rng = np.random.default_rng(0)
    # frames of different sizes and orders through the same graph
    for n in (len(d), 1000, 1, 0, 2500):
        sel = make_descs(d["pos"][rng.permutation(len(d))[:n]], 12) if n else d[:0]
        rec, tot = fb.build(sel)
        if n == 0:
            assert int(tot[0]) == 0 and int(tot[1]) == 0
            continue
        want = direct_build(ctx, sel, vcap, icap)
        np.testing.assert_array_equal(tot[:3], want.totals[:3])
        np.testing.assert_array_equal(rec, want.records)
        verts, norms, inds = fb.mesh(int(tot[0]), int(tot[1]))
        np.testing.assert_array_equal(inds, want.inds)
        np.testing.assert_array_equal(verts, want.verts)
        np.testing.assert_array_equal(norms, want.normals)
    # a new seed: the graph is recaptured and updated in place
    q = p.copy()
    q.seed = 9
    fb.set_params(q)
    sel = d[:1500]
    rec, tot = fb.build(sel)
    want = direct_build(ctx, sel, vcap, icap)
    np.testing.assert_array_equal(rec, want.records)
    # a change of launch shape (exact build, another kernel): re-instantiated
    q2 = q.copy()
    q2.math_mode = abi.UWW_MATH_EXACT
    fb.set_params(q2)
    rec, tot = fb.build(sel)
    want = direct_build(ctx, sel, vcap, icap)
    np.testing.assert_array_equal(rec, want.records)
    fb.close()


def test_frame_graph_recaptures_after_work_buffers_grow(ctx_factory):
    """A larger build on the same context reallocates the look-back words and
    the global scratch the captured graph refers to; the next frame launch
    recaptures the graph instead of using the freed buffers."""
    p, d = workloads.uniform_grid(seed=3, outputs=OUT)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    vcap, icap = 1 << 20, 1 << 22
    fb = FrameBuilder(ctx, 512, 12, vcap, icap)
    sel = d[:512]
    rec0, tot0 = fb.build(sel)
    # 8192 chunks (more look-back words) and 24-cell chunks (global scratch)
    big = make_descs(np.concatenate([d["pos"], d["pos"] + np.array([0, 0, 16], np.int32)]), 12)
    direct_build(ctx, big, 1 << 21, 1 << 23)
    direct_build(ctx, make_descs(d["pos"][:64], 24), 1 << 21, 1 << 23)
    rec, tot = fb.build(sel)
    np.testing.assert_array_equal(rec, rec0)
    np.testing.assert_array_equal(tot[:3], tot0[:3])
    want = direct_build(ctx, sel, vcap, icap)
    np.testing.assert_array_equal(rec, want.records)
    fb.close()


def test_frame_graph_rejects_a_count_above_its_maximum(ctx_factory):
    p, d = workloads.uniform_grid(seed=0)
    ctx = ctx_factory(p)
    fb = FrameBuilder(ctx, 16, 12, 1 << 16, 1 << 18, want_normals=False)
    fb.h_count.array[0] = 17
    assert abi.lib().uww_frame_launch(C.c_void_p(fb.handle)) == abi.UWW_ERR_INVALID_ARG
    fb.close()


def test_tunings_do_not_change_the_output(ctx_factory):
    p, d = workloads.mixed_lod(seed=1, n=256, outputs=OUT)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    base = direct_build(ctx, d, 1 << 21, 1 << 23)
    for th, bps, sc in [(64, 2, 0), (128, 1, 12), (192, 0, 24), (320, 0, 0), (512, 1, 12)]:
        ctx.set_tuning(threads=th, blocks_per_sm=bps, smem_cells=sc)
        got = direct_build(ctx, d, 1 << 21, 1 << 23)
        np.testing.assert_array_equal(got.records, base.records, err_msg=str((th, bps, sc)))
        np.testing.assert_array_equal(got.inds, base.inds)
        np.testing.assert_array_equal(got.verts, base.verts)
        np.testing.assert_array_equal(got.normals, base.normals)
    ctx.set_tuning()


def test_autotune_picks_caches_and_reuses(ctx_factory, tmp_path):
    p, d = workloads.mixed_lod(seed=0, n=512, outputs=OUT)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    vcap, icap = 1 << 21, 1 << 23
    d_desc = ctx.upload(d)
    bufs = [DeviceArray(vcap * 24), DeviceArray(vcap * 12), DeviceArray(icap * 4), DeviceArray(len(d) * 32),
            DeviceArray(32)]
    out = abi.MeshOut(bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, None, None, bufs[3].ptr, bufs[4].ptr, vcap, icap, 0, 0)
    cache = tmp_path / "tune.txt"
    t1, us1 = autotune(ctx, d_desc, len(d), 48, out, str(cache))
    assert us1 > 0 and t1.threads > 0 and t1.blocks_per_sm > 0
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and ",48:" in lines[0] and "oct6" in lines[0]
    # the context now runs with the tuning; a second call hits the cache
    got = abi.Tuning()
    abi.check(abi.lib().uww_ctx_get_tuning(ctx.h, C.byref(got)))
    assert (got.threads, got.blocks_per_sm, got.smem_cells) == (t1.threads, t1.blocks_per_sm, t1.smem_cells)
    t2, us2 = autotune(ctx, d_desc, len(d), 48, out, str(cache))
    assert (t2.threads, t2.blocks_per_sm, t2.smem_cells) == (t1.threads, t1.blocks_per_sm, t1.smem_cells)
    assert us2 == pytest.approx(us1, rel=1e-3)
    assert len(cache.read_text().splitlines()) == 1


def test_frame_graph_with_slabs_matches_direct_builds(ctx_factory):
    """The uneven-LOD world (24^3 and 48^3 chunks built as slabs) through a
    captured frame graph, with frames of different sizes read from the device
    count: the same records and mesh as direct builds."""
    p, d = workloads.mixed_lod(seed=4, outputs=OUT)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    assert ctx.launch_shape(len(d), 48).slabs_per_chunk > 1
    vcap, icap = 1 << 20, 1 << 22
    fb = FrameBuilder(ctx, len(d), 48, vcap, icap)
    rng = np.random.default_rng(1)
    for n in (len(d), 700, 3):
        idx = rng.permutation(len(d))[:n]
        sel = make_descs(d["pos"][idx], d["cells"][idx])
        rec, tot = fb.build(sel)
        want = direct_build(ctx, sel, vcap, icap)
        np.testing.assert_array_equal(tot[:3], want.totals[:3])
        np.testing.assert_array_equal(rec, want.records)
        verts, norms, inds = fb.mesh(int(tot[0]), int(tot[1]))
        np.testing.assert_array_equal(inds, want.inds)
        np.testing.assert_array_equal(verts, want.verts)
        np.testing.assert_array_equal(norms, want.normals)
    fb.close()
