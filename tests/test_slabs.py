"""Chunks above 16 cells per edge built as x slabs by the split build.

The split build builds every chunk of 17..63 cells per edge as slabs of a
few cell layers, one CTA each (any batch whose samples are computed, not
read); a slab's references to vertices of the previous slab's last layer go
through that slab's seam.  Per-cell cases, samples and per-vertex edge ids
(the adjoint's forward) come from the slabs too.  The output must be the
chunk's, bit for bit: against the F32 oracle (parity build, chunk.rs:135-264
with perlin_util.rs:6-29), and against the single pipelined kernel, which
builds each chunk whole (fast build).  Covered: the uneven-LOD batch
(12^3 / 24^3 / 48^3), both dedup modes, odd sizes (17, 31 and 63 cells: the
last slab shorter than the others), dense slabs (more active cells than a
slab's active-cell list holds, so that pass 1 walks the cell columns), and
batches whose output exceeds the capacities, so that slabs find no room in
the staging buffers and the emission kernel builds them again in place.
"""
import os

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.adjoint import Adjoint
from underwaterworld_gb300.chunk import make_descs

from helpers import assert_batches_equal, relayout

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
COLOR_NORMALS = abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS


def caps(ref):
    return max(int(ref.totals[0]), 1), max(int(ref.totals[1]), 1)


def assert_same_bytes(a, b):
    np.testing.assert_array_equal(a.records, b.records)
    np.testing.assert_array_equal(a.totals, b.totals)
    np.testing.assert_array_equal(a.inds, b.inds)
    np.testing.assert_array_equal(a.verts.view(np.uint32), b.verts.view(np.uint32))
    if a.normals is not None:
        np.testing.assert_array_equal(a.normals.view(np.uint32), b.normals.view(np.uint32))


def odd_sizes(seed=0, n=96):
    """Chunks of 17, 31 and 63 cells around the surface of the mixed-LOD world."""
    p, _ = workloads.mixed_lod(seed=seed, outputs=COLOR_NORMALS)
    rng = np.random.default_rng(seed)
    pos = np.stack([rng.integers(-8, 8, n), rng.integers(-8, 8, n), rng.integers(-2, 2, n)], -1)
    cells = rng.choice(np.array([12, 17, 31, 63]), size=n)
    return p, make_descs(pos, cells)


# a slab's active-cell list holds this many cells; a slab with more walks its
# cell columns in pass 1 instead
SLAB_LIST_CELLS = 2048


def dense_slabs(seed=0):
    """Chunks of 48, 24, 63, 17, 12 and 31 cells in a short-wavelength 6-octave
    fBm (0.3 per world unit) with no depth bias: about 2,100 to 3,900 active
    cells in most slabs of every size, a few below the list's capacity."""
    p = workloads.fbm_params(seed, 6, 0.3, 0.0, 0.0, 0.0, COLOR_NORMALS)
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [2, 0, 0], [0, 2, 0]])
    return p, make_descs(pos, np.array([48, 24, 63, 17, 12, 31]))


def test_mixed_batch_takes_the_slab_build(ctx_factory):
    p, d = workloads.mixed_lod(seed=0, outputs=COLOR_NORMALS)
    ctx = ctx_factory(p)
    s = ctx.launch_shape(len(d), 48)
    assert s.build == abi.UWW_BUILD_SPLIT and s.slabs_per_chunk > 1 and s.threads == 256
    # per-cell cases as well (the planning kernel then decides nothing)
    q = p.copy()
    q.outputs = COLOR_NORMALS | abi.UWW_OUT_CASES
    s = ctx_factory(q).launch_shape(len(d), 48)
    assert s.build == abi.UWW_BUILD_SPLIT and s.slabs_per_chunk > 1
    ctx.set_tuning(options=abi.UWW_TUNE_PIPELINED)
    assert ctx.launch_shape(len(d), 48).build == abi.UWW_BUILD_PIPELINED
    ctx.set_tuning(options=0)


@pytest.mark.parametrize("dedup", [abi.UWW_DEDUP_ORIENTED, abi.UWW_DEDUP_EDGE])
def test_slab_build_bit_exact_against_the_oracle(ctx_factory, oracle, dedup):
    p, d = workloads.mixed_lod(seed=0, outputs=COLOR_NORMALS)
    p.dedup_mode = dedup
    if dedup == abi.UWW_DEDUP_EDGE:
        d = relayout(d[:768])
    ref = oracle.build_chunks(p, d, precision=oracle.F32, threads=THREADS)
    ctx = ctx_factory(p)
    assert ctx.launch_shape(len(d), 48).slabs_per_chunk > 1
    got = ctx.build_chunks_device(d, *caps(ref))
    assert got.status == abi.UWW_OK
    assert_batches_equal(got, ref)
    big = d["cells"] > 16
    assert (ref.records["flags"][big] & abi.UWW_CHUNK_HAS_MESH).sum() > 20


def test_odd_sizes_bit_exact_against_the_oracle(ctx_factory, oracle):
    p, d = odd_sizes()
    ref = oracle.build_chunks(p, d, precision=oracle.F32, threads=THREADS)
    got = ctx_factory(p).build_chunks_device(d, *caps(ref))
    assert got.status == abi.UWW_OK
    assert_batches_equal(got, ref)
    assert (ref.records["flags"][d["cells"] == 63] & abi.UWW_CHUNK_HAS_MESH).sum() > 3


@pytest.mark.parametrize("dedup", [abi.UWW_DEDUP_ORIENTED, abi.UWW_DEDUP_EDGE])
def test_dense_slabs_bit_exact_against_the_oracle(ctx_factory, oracle, dedup):
    p, d = dense_slabs()
    p.dedup_mode = dedup
    ref = oracle.build_chunks(p, d, precision=oracle.F32, threads=THREADS)
    ctx = ctx_factory(p)
    # the 48^3 chunk averages more active cells per slab than the list holds
    slabs = ctx.launch_shape(1, 48).slabs_per_chunk
    assert slabs > 1 and int(ref.records["num_active_cells"][0]) > SLAB_LIST_CELLS * slabs
    got = ctx.build_chunks_device(d, *caps(ref))
    assert got.status == abi.UWW_OK
    assert_batches_equal(got, ref)


@pytest.mark.parametrize("frac", [1.0, 0.6])
def test_dense_slabs_match_the_pipelined_build(ctx_factory, frac):
    """Fast build, dense slabs: byte-equal to the pipelined build; at 60 % of
    the output's size the staging buffers run out, so the emission kernel
    builds dense slabs again (walking their columns), and the chunks that fit
    are identical to the full build's."""
    p, d = dense_slabs(seed=1)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    full = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    assert full.status == abi.UWW_OK
    vcap, icap = int(full.totals[0] * frac), int(full.totals[1] * frac)
    slabs = ctx.build_chunks_device(d, vcap, icap)
    ctx.set_tuning(options=abi.UWW_TUNE_PIPELINED)
    piped = ctx.build_chunks_device(d, vcap, icap)
    ctx.set_tuning(options=0)
    if frac == 1.0:
        assert slabs.status == abi.UWW_OK and piped.status == abi.UWW_OK
        assert_same_bytes(slabs, piped)
        assert_same_bytes(slabs, full)
        return
    assert slabs.status == abi.UWW_ERR_CAPACITY and piped.status == abi.UWW_ERR_CAPACITY
    np.testing.assert_array_equal(slabs.records, piped.records)
    np.testing.assert_array_equal(slabs.totals[:3], piped.totals[:3])
    ok = (slabs.records["flags"] & abi.UWW_CHUNK_OVERFLOW) == 0
    assert ok[0] and (~ok).sum() > 0
    rec = full.records
    for i in np.nonzero(ok & (rec["num_inds"] > 0))[0]:
        v0, nv = rec["vert_offset"][i], rec["num_verts"][i]
        i0, ni = rec["ind_offset"][i], rec["num_inds"][i]
        np.testing.assert_array_equal(slabs.inds[i0:i0 + ni], full.inds[i0:i0 + ni])
        np.testing.assert_array_equal(slabs.verts[v0:v0 + nv].view(np.uint32), full.verts[v0:v0 + nv].view(np.uint32))
        np.testing.assert_array_equal(slabs.normals[v0:v0 + nv].view(np.uint32),
                                      full.normals[v0:v0 + nv].view(np.uint32))


@pytest.mark.parametrize("seed", [0, 5])
def test_slab_and_pipelined_builds_give_the_same_bytes(ctx_factory, seed):
    p, d = workloads.mixed_lod(seed=seed, outputs=COLOR_NORMALS)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    slabs = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    ctx.set_tuning(options=abi.UWW_TUNE_PIPELINED)
    piped = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    ctx.set_tuning(options=0)
    again = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    for b in (slabs, piped, again):
        assert b.status == abi.UWW_OK
    assert_same_bytes(slabs, piped)
    assert_same_bytes(slabs, again)


def test_odd_sizes_fast_build_matches_the_pipelined_build(ctx_factory):
    p, d = odd_sizes(seed=1)
    p.math_mode = abi.UWW_MATH_FAST
    p.dedup_mode = abi.UWW_DEDUP_EDGE
    ctx = ctx_factory(p)
    slabs = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    ctx.set_tuning(options=abi.UWW_TUNE_PIPELINED)
    piped = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    ctx.set_tuning(options=0)
    assert slabs.status == abi.UWW_OK and piped.status == abi.UWW_OK
    assert_same_bytes(slabs, piped)


@pytest.mark.parametrize("frac", [0.5, 0.97])
def test_slabs_without_staging_room(ctx_factory, frac):
    """Capacities below the batch's output: the staging buffers (as large as the
    outputs) run out, so some slabs are built again by the emission kernel;
    chunks that fit are written as the pipelined build writes them, the rest
    are flagged, and nothing lands past the capacities."""
    p, d = workloads.mixed_lod(seed=3, outputs=COLOR_NORMALS)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    full = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    assert full.status == abi.UWW_OK
    vcap, icap = int(full.totals[0] * frac), int(full.totals[1] * frac)
    small = ctx.build_chunks_device(d, vcap, icap)
    ctx.set_tuning(options=abi.UWW_TUNE_PIPELINED)
    piped = ctx.build_chunks_device(d, vcap, icap)
    ctx.set_tuning(options=0)
    assert small.status == abi.UWW_ERR_CAPACITY and piped.status == abi.UWW_ERR_CAPACITY
    np.testing.assert_array_equal(small.records, piped.records)
    np.testing.assert_array_equal(small.totals[:3], piped.totals[:3])
    ok = (small.records["flags"] & abi.UWW_CHUNK_OVERFLOW) == 0
    assert ok.sum() > 100 and (~ok).sum() > 0
    rec = full.records
    for i in np.nonzero(ok & (rec["num_inds"] > 0))[0]:
        v0, nv = rec["vert_offset"][i], rec["num_verts"][i]
        i0, ni = rec["ind_offset"][i], rec["num_inds"][i]
        np.testing.assert_array_equal(small.inds[i0:i0 + ni], full.inds[i0:i0 + ni])
        np.testing.assert_array_equal(small.verts[v0:v0 + nv].view(np.uint32), full.verts[v0:v0 + nv].view(np.uint32))
        np.testing.assert_array_equal(small.normals[v0:v0 + nv].view(np.uint32),
                                      full.normals[v0:v0 + nv].view(np.uint32))


@pytest.mark.parametrize("cells", [24, 16])
def test_forward_with_edge_ids_matches_the_pipelined_build(ctx_factory, cells):
    """uww_forward (records, vertices, cases and per-vertex edge ids) through the
    split build -- slabs for 24^3, whole chunks for 16^3 -- against the
    pipelined build, byte for byte (fast build)."""
    p, d = workloads.adjoint_batch(seed=0, side=6, cells=cells)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    assert ctx.launch_shape(len(d), cells).build == abi.UWW_BUILD_SPLIT
    a = Adjoint(ctx, d, 1 << 20, 1 << 22)
    a.forward()
    split = a.fetch_forward()
    ctx.set_tuning(options=abi.UWW_TUNE_PIPELINED)
    a.forward()
    piped = a.fetch_forward()
    ctx.set_tuning(options=0)
    assert int(split["totals"][0]) > 1000
    for k in ("totals", "records", "edge_ids", "cases"):
        np.testing.assert_array_equal(split[k], piped[k], err_msg=k)
    np.testing.assert_array_equal(split["verts"].view(np.uint32), piped["verts"].view(np.uint32))


@pytest.mark.parametrize("shift", [0, 4])
def test_host_buffers_with_slabs(ctx_factory, shift):
    """uww_build_chunks_host into page-locked buffers on an uneven-LOD batch
    (slabs): the emission's direct stores (aligned buffers) or the sized copy
    (buffers shifted by 4 bytes) give the device build's records, vertices,
    normals and indices."""
    import ctypes as C
    from underwaterworld_gb300.chunk import HostArray
    p, d = workloads.mixed_lod(seed=6, outputs=COLOR_NORMALS)
    p.math_mode = abi.UWW_MATH_FAST
    d = relayout(d[:512])
    ctx = ctx_factory(p)
    want = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    assert want.status == abi.UWW_OK
    n = len(d)
    vcap, icap = int(want.totals[0]) + 3, int(want.totals[1]) + 5
    keep = []

    def host(shape, dtype):
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        h = HostArray((nbytes + 16,), np.uint8)
        keep.append(h)
        return h.ptr + shift, h.array[shift:shift + nbytes].view(dtype).reshape(shape)

    pv, hv = host((vcap,), abi.VERT_COLOR_DTYPE)
    pn, hn = host((vcap, 3), np.float32)
    pi, hi = host((icap,), np.uint32)
    pr, hr = host((n,), abi.CHUNK_RECORD_DTYPE)
    tot = np.zeros(4, np.uint64)
    out = abi.MeshOut(pv, pn, pi, None, None, pr, tot.ctypes.data, vcap, icap, 0, 0)
    h_desc = HostArray((n,), abi.CHUNK_DESC_DTYPE)
    h_desc.array[:] = d
    abi.check(abi.lib().uww_build_chunks_host(ctx.h, C.c_void_p(h_desc.ptr), n, C.byref(out)), "host build")
    nv, ni = int(tot[0]), int(tot[1])
    np.testing.assert_array_equal(tot[:3], want.totals[:3])
    np.testing.assert_array_equal(hr, want.records)
    np.testing.assert_array_equal(hv[:nv].view(np.uint32), want.verts.view(np.uint32))
    np.testing.assert_array_equal(hn[:nv].view(np.uint32), want.normals.view(np.uint32))
    np.testing.assert_array_equal(hi[:ni], want.inds)
