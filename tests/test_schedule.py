"""The scheduler feed (World::update_nearby, world.rs:148-234): candidate
positions, frustum classes and GenPrio order on the GPU against the CPU
restatement, exactly (same f32 operation order)."""
import ctypes as C

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import make_descs
from underwaterworld_gb300.schedule import Scheduler, schedule_params

pytestmark = pytest.mark.gpu


def cameras(seed, n):
    r = np.random.default_rng(seed)
    for _ in range(n):
        sub = r.uniform([-60, -60, -30], [60, 60, 30]).astype(np.float32)
        bearing = r.normal(size=3).astype(np.float32)
        bearing[2] *= 0.3
        eye = sub - 6.0 * bearing / np.linalg.norm(bearing) + np.array([0, 0, 2], np.float32)
        yield sub, eye, sub + bearing


@pytest.mark.parametrize("with_known", [False, True])
def test_schedule_matches_the_oracle(ctx_factory, oracle, with_known):
    p, _ = workloads.reference_grid(outputs=abi.UWW_OUT_CASES)
    ctx = ctx_factory(p)
    known = None
    kd = kr = None
    if with_known:
        # the chunks already built: a slab around the origin
        g = np.arange(-3, 3)
        pos = np.stack(np.meshgrid(g, g, np.arange(-2, 3), indexing="ij"), -1).reshape(-1, 3)
        kd = make_descs(pos, 12)
        b = ctx.build_chunks_device(kd, 1 << 20, 1 << 22)
        kr = b.records
        d_kd, d_kr = ctx.upload(kd), ctx.upload(kr)
        size = 1 << int(2 * len(kd) - 1).bit_length()
        from underwaterworld_gb300.chunk import DeviceArray
        d_t = DeviceArray(size * 4)
        abi.check(abi.lib().uww_chunk_index(ctx.h, C.c_void_p(d_kd.ptr), len(kd), C.c_void_p(d_t.ptr), size))
        known = (d_kd.ptr, d_kr.ptr, d_t.ptr, size)
        assert (kr["flags"] & abi.UWW_CHUNK_HAS_MESH).any()
    sch = Scheduler(ctx)
    n_render = 0
    for sub, eye, tgt in cameras(7 + with_known, 12):
        sub[:2] *= 0.2 if with_known else 1.0
        sp = schedule_params(sub, eye, tgt)
        sch.run(sp, known)
        gen, ren, counts = sch.fetch()
        want_gen, want_ren = oracle.schedule_chunks(p, sp, kd, kr)
        assert int(counts[0]) == len(want_gen) and int(counts[1]) == len(want_ren)
        np.testing.assert_array_equal(gen, want_gen)
        np.testing.assert_array_equal(ren, want_ren)
        n_render += len(ren)
    if with_known:
        assert n_render > 0


def test_generation_list_feeds_the_build(ctx_factory, oracle):
    """The generation list is the batched build's input as is."""
    p, _ = workloads.reference_grid(outputs=abi.UWW_OUT_COLOR)
    p.math_mode = abi.UWW_MATH_EXACT
    ctx = ctx_factory(p)
    sch = Scheduler(ctx)
    sub, eye, tgt = next(cameras(3, 1))
    sch.run(schedule_params(sub, eye, tgt))
    gen, _, counts = sch.fetch()
    assert len(gen) > 100
    b = ctx.build_chunks_device(gen, 1 << 21, 1 << 23)
    want = oracle.build_chunks(p, gen, precision=oracle.F32)
    np.testing.assert_array_equal(b.records, want.records)
    np.testing.assert_array_equal(b.inds, want.inds)
