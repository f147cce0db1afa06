"""The batched builds' bounded waits, made to run out on purpose.

The device-wide prefix sum of the batched build (a decoupled look-back over
the work-queue order) makes each chunk wait for the words its predecessors
publish.  Every such wait is bounded by the context's spin limit; a wait that
gives up raises UWW_ERRFLAG_TIMEOUT, saturates the chunk's prefix (so the
chunk is flagged as an overflow and not written) and the build carries on.

UWW_TEST_WITHHOLD_FIRST makes the first chunk of the batch never publish its
prefix -- a flag that nothing sets -- and a short spin limit makes the waits
behind it run out quickly.  Nothing faults and nothing hangs: the launch ends
by itself, the call reports UWW_ERR_TIMEOUT, no byte outside the output
capacities changes, and the same context then builds the batch correctly at
the default limit.  (The reference has no such path: a failed chunk build
panics, state.rs:106.)

The split build waits in one place: each emission CTA, before its first
store, for the records of every tile.  UWW_TEST_WITHHOLD_RECORDS makes the
first tile's records never be announced; the waits run out, the build
reports UWW_ERR_TIMEOUT and stores no vertex, normal or index, and again the
context recovers.
"""
import ctypes as C

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import DeviceArray, totals_status

from helpers import assert_batches_equal, relayout

pytestmark = pytest.mark.gpu

GUARD = 4096  # bytes past every capacity that must stay untouched
SHORT_SPIN = 100_000  # cycles, about 50 us at 2 GHz


def set_tuning(ctx, spin_limit, test_flags):
    t = abi.Tuning()
    abi.check(abi.lib().uww_ctx_get_tuning(ctx.h, C.byref(t)))
    t.spin_limit, t.test_flags = spin_limit, test_flags
    abi.check(abi.lib().uww_ctx_set_tuning(ctx.h, C.byref(t)))


@pytest.mark.parametrize("outputs", [abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS,
                                     abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS | abi.UWW_OUT_CASES])
def test_withheld_prefix_times_out_and_the_context_recovers(ctx_factory, oracle, outputs):
    # colour + normals: a planned batch, whose work queue holds only the
    # chunks the depth bias does not decide (the others' records follow the
    # look-back of the queued chunk before them); with cases, every chunk is
    # queued
    p, d = workloads.uniform_grid(seed=2, outputs=outputs)
    p.math_mode = abi.UWW_MATH_FAST
    n = len(d)
    ref = oracle.build_chunks(p, d, precision=oracle.F32, threads=8)
    vcap, icap = int(ref.totals[0]) + 64, int(ref.totals[1]) + 64
    ncells = int((d["cells"].astype(np.int64) ** 3).sum())
    ctx = ctx_factory(p)
    d_desc = ctx.upload(d)
    sizes = {"verts": vcap * 24, "normals": vcap * 12, "inds": icap * 4, "records": n * 32, "totals": 32,
             "cases": ncells}
    bufs = {k: DeviceArray(v + GUARD) for k, v in sizes.items()}
    guard = np.full(max(sizes.values()) + GUARD, 0xAB, np.uint8)
    for k, b in bufs.items():
        abi.check(abi.lib().uww_memcpy(ctx.h, C.c_void_p(b.ptr), guard.ctypes.data_as(C.c_void_p), b.nbytes, abi.H2D))
    want_cases = bool(outputs & abi.UWW_OUT_CASES)
    out = abi.MeshOut(bufs["verts"].ptr, bufs["normals"].ptr, bufs["inds"].ptr,
                      bufs["cases"].ptr if want_cases else None, None, bufs["records"].ptr, bufs["totals"].ptr,
                      vcap, icap, ncells if want_cases else 0, 0)

    set_tuning(ctx, SHORT_SPIN, abi.UWW_TEST_WITHHOLD_FIRST)
    abi.check(abi.lib().uww_build_chunks(ctx.h, C.c_void_p(d_desc.ptr), n, 12, C.byref(out)), "launch")
    ctx.sync()  # the launch ended by itself
    tot = ctx.download(bufs["totals"], (4,), np.uint64)
    assert totals_status(tot) == abi.UWW_ERR_TIMEOUT, tot
    assert int(tot[3]) & abi.UWW_ERRFLAG_TIMEOUT
    rec = ctx.download(bufs["records"], (n,), abi.CHUNK_RECORD_DTYPE)
    # the chunks up to and including the first chunk of the work queue (and,
    # with colour + normals, the chunks the depth bias decides right after
    # it) have exact prefixes; every later chunk has a saturated prefix:
    # flagged as an overflow, not written
    over = (rec["flags"] & abi.UWW_CHUNK_OVERFLOW) != 0
    k = int(np.argmax(over))
    assert 1 <= k < n // 4 and not over[:k].any() and over[k:].all(), k
    assert int(tot[2]) == n - k
    np.testing.assert_array_equal(rec["num_inds"], ref.records["num_inds"])
    for name, b in bufs.items():
        back = ctx.download(b, (b.nbytes,), np.uint8)
        assert np.all(back[sizes[name]:] == 0xAB), f"{name}: bytes written past the capacity"

    # the same context, default limit, no injection: the batch builds correctly
    set_tuning(ctx, 0, 0)
    q = p.copy()
    q.math_mode = abi.UWW_MATH_EXACT
    ctx.set_params(q)
    got = ctx.build_chunks_device(d, vcap, icap)
    assert got.status == abi.UWW_OK
    assert_batches_equal(got, ref)


def test_spin_limit_and_test_flags_are_validated(ctx_factory):
    p, _ = workloads.uniform_grid(seed=0)
    ctx = ctx_factory(p)
    t = abi.Tuning()
    abi.check(abi.lib().uww_ctx_get_tuning(ctx.h, C.byref(t)))
    assert (t.spin_limit, t.test_flags) == (0, 0)
    bad = abi.Tuning()
    C.pointer(bad)[0] = t
    bad.spin_limit = -1
    assert abi.lib().uww_ctx_set_tuning(ctx.h, C.byref(bad)) == abi.UWW_ERR_INVALID_ARG
    bad.spin_limit, bad.test_flags = 0, 4
    assert abi.lib().uww_ctx_set_tuning(ctx.h, C.byref(bad)) == abi.UWW_ERR_INVALID_ARG
    ctx.set_tuning(threads=128)  # the launch-shape setter keeps the spin limit
    set_tuning(ctx, 5000, 0)
    ctx.set_tuning(threads=160)
    abi.check(abi.lib().uww_ctx_get_tuning(ctx.h, C.byref(t)))
    assert (t.threads, t.spin_limit, t.test_flags) == (160, 5000, 0)


@pytest.mark.parametrize("world", ["uniform", "slabs"])
def test_withheld_records_time_out_and_the_context_recovers(ctx_factory, oracle, world):
    """The split build's records wait runs out (records withheld): whole chunks
    on the uniform grid, and a batch of the uneven-LOD world whose 24^3 and
    48^3 chunks are built as slabs."""
    if world == "uniform":
        p, d = workloads.uniform_grid(seed=4, outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS)
    else:
        p, d = workloads.mixed_lod(seed=4, outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS)
        d = relayout(d[:384])
    max_cells = int(d["cells"].max())
    p.math_mode = abi.UWW_MATH_FAST
    n = len(d)
    ref = oracle.build_chunks(p, d, precision=oracle.F32, threads=8)
    vcap, icap = int(ref.totals[0]) + 64, int(ref.totals[1]) + 64
    ctx = ctx_factory(p)
    clean = ctx.build_chunks_device(d, vcap, icap)  # the same fast build, nothing withheld
    assert clean.status == abi.UWW_OK
    d_desc = ctx.upload(d)
    sizes = {"verts": vcap * 24, "normals": vcap * 12, "inds": icap * 4, "records": n * 32, "totals": 32}
    bufs = {k: DeviceArray(v + GUARD) for k, v in sizes.items()}
    guard = np.full(max(sizes.values()) + GUARD, 0xAB, np.uint8)
    for k, b in bufs.items():
        abi.check(abi.lib().uww_memcpy(ctx.h, C.c_void_p(b.ptr), guard.ctypes.data_as(C.c_void_p), b.nbytes, abi.H2D))
    out = abi.MeshOut(bufs["verts"].ptr, bufs["normals"].ptr, bufs["inds"].ptr, None, None, bufs["records"].ptr,
                      bufs["totals"].ptr, vcap, icap, 0, 0)

    if world == "slabs":
        assert ctx.launch_shape(n, max_cells).slabs_per_chunk > 1
    set_tuning(ctx, SHORT_SPIN, abi.UWW_TEST_WITHHOLD_RECORDS)
    abi.check(abi.lib().uww_build_chunks(ctx.h, C.c_void_p(d_desc.ptr), n, max_cells, C.byref(out)), "launch")
    ctx.sync()  # the launch ended by itself
    tot = ctx.download(bufs["totals"], (4,), np.uint64)
    assert totals_status(tot) == abi.UWW_ERR_TIMEOUT, tot
    # the records were written (only not announced) and the totals are right
    np.testing.assert_array_equal(tot[:2], clean.totals[:2])
    rec = ctx.download(bufs["records"], (n,), abi.CHUNK_RECORD_DTYPE)
    np.testing.assert_array_equal(rec, clean.records)
    # no vertex, normal or index stored, nothing past any capacity
    for name in ("verts", "normals", "inds"):
        back = ctx.download(bufs[name], (bufs[name].nbytes,), np.uint8)
        assert np.all(back == 0xAB), f"{name}: stored although the records were never announced"
    back = ctx.download(bufs["records"], (bufs["records"].nbytes,), np.uint8)
    assert np.all(back[sizes["records"]:] == 0xAB)

    # the same context, default limit, no injection: the batch builds correctly
    set_tuning(ctx, 0, 0)
    q = p.copy()
    q.math_mode = abi.UWW_MATH_EXACT
    ctx.set_params(q)
    got = ctx.build_chunks_device(d, vcap, icap)
    assert got.status == abi.UWW_OK
    assert_batches_equal(got, ref)
