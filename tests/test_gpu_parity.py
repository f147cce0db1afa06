"""CUDA chunk builder vs the CPU oracle, through the C ABI.

Parity build (UWW_MATH_EXACT): case indices, counts, flags, offsets, index
buffers and vertex positions bit-exact; colours within COLOR_ATOL (powf);
normals within NORMAL_ATOL.  Fast build: flipped cells and vertex error
against the f64 oracle, reported and bounded; colours and normals against
the F32 oracle, bounded.
"""
import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import Chunk, make_descs

from helpers import (assert_batches_equal, assert_records_equal, flipped_cells, load_golden, params_for_samples,
                     relayout)

pytestmark = pytest.mark.gpu

ALL = abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS | abi.UWW_OUT_CASES


def caps(ref):
    return max(int(ref.totals[0]), 1), max(int(ref.totals[1]), 1)


@pytest.fixture(params=["split", "pipelined"])
def ctx_factory(request, ctx_factory):
    """Every test here runs twice: with the default batched build (the split
    build wherever every chunk fits a shared-memory workspace) and with the
    single pipelined kernel (UWW_TUNE_PIPELINED)."""
    if request.param == "split":
        return ctx_factory

    def make(params=None):
        c = ctx_factory(params)
        c.set_tuning(options=abi.UWW_TUNE_PIPELINED)
        return c

    return make


@pytest.mark.parametrize("name", ["single_cell", "single_cell_random", "grids"])
def test_known_answers_from_samples(ctx_factory, oracle, name):
    g = load_golden(name)
    p = params_for_samples(g["iso_level"])
    ctx = ctx_factory(p)
    b = ctx.build_chunks_device(g["descs"], int(g["num_verts"].sum()) + 1, int(g["num_inds"].sum()) + 1,
                                samples_in=g["samples"])
    assert b.status == abi.UWW_OK
    np.testing.assert_array_equal(b.records["num_verts"], g["num_verts"])
    np.testing.assert_array_equal(b.records["num_inds"], g["num_inds"])
    np.testing.assert_array_equal(b.inds, g["inds"])
    np.testing.assert_array_equal(b.cases, g["cases"])
    np.testing.assert_array_equal(b.verts["pos"], g["verts"])
    np.testing.assert_allclose(b.verts["color"], g["colors"], rtol=0, atol=2e-6)


@pytest.mark.parametrize("iso", [-0.1, 0.0])
@pytest.mark.parametrize("dedup", [abi.UWW_DEDUP_ORIENTED, abi.UWW_DEDUP_EDGE])
def test_reference_grid_bit_exact(ctx_factory, oracle, iso, dedup):
    p, d = workloads.reference_grid(iso_level=iso, outputs=ALL)
    p.dedup_mode = dedup
    ref = oracle.build_chunks(p, d, precision=oracle.F32)
    ctx = ctx_factory(p)
    got = ctx.build_chunks_device(d, *caps(ref))
    assert got.status == abi.UWW_OK
    assert_batches_equal(got, ref)


def test_host_path_equals_device_path(ctx_factory, oracle):
    p, d = workloads.reference_grid(outputs=ALL)
    ctx = ctx_factory(p)
    ref = oracle.build_chunks(p, d)
    a = ctx.build_chunks(d, *caps(ref))
    b = ctx.build_chunks_device(d, *caps(ref))
    assert a.status == abi.UWW_OK
    assert_batches_equal(a, b)
    assert_batches_equal(a, ref)


def test_uniform_grid_subset_bit_exact(ctx_factory, oracle):
    p, d = workloads.uniform_grid(seed=3, outputs=ALL)
    # the z-layers that straddle the surface, plus blank ones above and below
    sel = relayout(d[(d["pos"][:, 0] < 6) & (d["pos"][:, 1] < 6)])
    ref = oracle.build_chunks(p, sel)
    got = ctx_factory(p).build_chunks_device(sel, *caps(ref))
    assert_batches_equal(got, ref)
    assert (ref.records["flags"] & abi.UWW_CHUNK_HAS_MESH).sum() > 10


@pytest.mark.parametrize("cells", [24, 48, 5, 1])
def test_other_lods_bit_exact(ctx_factory, oracle, cells):
    p, _ = workloads.uniform_grid(seed=1, outputs=ALL)
    pos = [(1, 2, 7), (3, 3, 8), (0, 5, 7), (2, 2, 2)]
    d = make_descs(pos, cells)
    ref = oracle.build_chunks(p, d)
    got = ctx_factory(p).build_chunks_device(d, *caps(ref))
    assert_batches_equal(got, ref)


def test_mixed_lod_batch_bit_exact(ctx_factory, oracle):
    p, d = workloads.mixed_lod(seed=2, outputs=ALL)
    sel = relayout(d[:96])
    ref = oracle.build_chunks(p, sel)
    got = ctx_factory(p).build_chunks_device(sel, *caps(ref))
    assert_batches_equal(got, ref)


def test_plain_per_chunk_launch_matches_batch(ctx_factory, oracle):
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS)
    ctx = ctx_factory(p)
    ref = oracle.build_chunks(p, d)
    for i in [0, 31, 62, 64, 100, 124]:
        ch = Chunk(tuple(d["pos"][i]))
        ch.build_full(ctx)
        v, n, ind = ref.chunk(i)
        assert ch.num_inds() == len(ind)
        assert ch.not_blank() == (len(ind) > 0)
        np.testing.assert_array_equal(ch.inds(), ind)
        np.testing.assert_array_equal(ch.verts()["pos"], v["pos"])
        np.testing.assert_allclose(ch.normals(), n, atol=1e-6)


def test_density_at_matches_oracle(ctx_factory, oracle):
    for p, lo, hi in [(workloads.reference_grid()[0], -40, 40), (workloads.uniform_grid(seed=4)[0], 0, 256)]:
        rng = np.random.default_rng(5)
        x = rng.uniform(lo, hi, (10000, 3)).astype(np.float32)
        np.testing.assert_array_equal(ctx_factory(p).density_at(x), oracle.density_at(p, x))


def test_iso_at_chunk_units(ctx_factory, oracle):
    p = abi.reference_params()
    ctx = ctx_factory(p)
    v = ctx.iso_at(0.5, -1.25, 0.75)
    assert v == oracle.density_at(p, np.array([[8.0, -20.0, 12.0]], np.float32))[0]


def test_capacity_overflow_then_regrow(ctx_factory, oracle):
    p, d = workloads.reference_grid(outputs=ALL)
    ctx = ctx_factory(p)
    ref = oracle.build_chunks(p, d)
    small = ctx.build_chunks_device(d, 1000, 3000)
    assert small.status == abi.UWW_ERR_CAPACITY
    np.testing.assert_array_equal(small.totals[:2], ref.totals[:2])
    assert int(small.totals[2]) > 0
    ok = (small.records["flags"] & abi.UWW_CHUNK_OVERFLOW) == 0
    np.testing.assert_array_equal(small.records["num_inds"], ref.records["num_inds"])
    # chunks that fitted were written correctly
    for i in np.nonzero(ok & (ref.records["num_inds"] > 0))[0]:
        v0, nv = ref.records["vert_offset"][i], ref.records["num_verts"][i]
        i0, ni = ref.records["ind_offset"][i], ref.records["num_inds"][i]
        np.testing.assert_array_equal(small.inds[i0:i0 + ni], ref.inds[i0:i0 + ni])
        np.testing.assert_array_equal(small.verts["pos"][v0:v0 + nv], ref.verts["pos"][v0:v0 + nv])
    big = ctx.build_chunks_device(d, int(small.totals[0]), int(small.totals[1]))
    assert big.status == abi.UWW_OK
    assert_batches_equal(big, ref)


def test_empty_blank_and_solid_batches(ctx_factory, oracle):
    p, d = workloads.reference_grid(outputs=ALL)
    ctx = ctx_factory(p)
    e = ctx.build_chunks_device(d[:0], 16, 16)
    assert e.totals[0] == 0 and e.totals[1] == 0
    for iso in (-50.0, 50.0):  # everything outside / everything inside
        q = p.copy()
        q.iso_level = iso
        ctx.set_params(q)
        b = ctx.build_chunks_device(d, 16, 16)
        ref = oracle.build_chunks(q, d)
        assert b.status == abi.UWW_OK and b.totals[0] == 0 and b.totals[1] == 0
        assert_records_equal(b.records, ref.records)
        np.testing.assert_array_equal(b.cases, ref.cases)
        expect = abi.UWW_CHUNK_EARLY_BLANK if iso < 0 else 0
        assert np.all(b.records["flags"] == expect)


def test_bad_descriptor_is_flagged_not_built(ctx_factory):
    p, d = workloads.reference_grid()
    ctx = ctx_factory(p)
    bad = d[:4].copy()
    bad["cells"][2] = 40  # above the max_cells the launch was given
    b = ctx.build_chunks_device(relayout(bad[[0, 1, 3]]), 5000, 20000)  # sanity: good chunks alone
    assert b.status == abi.UWW_OK
    import ctypes as C
    from underwaterworld_gb300.chunk import DeviceArray
    d_desc = ctx.upload(bad)
    d_rec, d_tot = DeviceArray(4 * 32), DeviceArray(32)
    d_v, d_i = DeviceArray(5000 * 24), DeviceArray(20000 * 4)
    out = abi.MeshOut(d_v.ptr, None, d_i.ptr, None, None, d_rec.ptr, d_tot.ptr, 5000, 20000)
    assert abi.lib().uww_build_chunks(ctx.h, C.c_void_p(d_desc.ptr), 4, 12, C.byref(out)) == abi.UWW_OK
    ctx.sync()
    tot = ctx.download(d_tot, (4,), np.uint64)
    assert int(tot[3]) & abi.UWW_ERRFLAG_BAD
    rec = ctx.download(d_rec, (4,), abi.CHUNK_RECORD_DTYPE)
    assert rec["num_inds"][2] == 0


def test_per_cell_outputs_are_range_checked(ctx_factory):
    """A cases buffer smaller than the descriptors' cell offsets need: no write past it."""
    import ctypes as C
    from underwaterworld_gb300.chunk import DeviceArray
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_CASES)
    ctx = ctx_factory(p)
    d = d[:8]
    d_desc = ctx.upload(d)
    d_rec, d_tot = DeviceArray(8 * 32), DeviceArray(32)
    d_v, d_i = DeviceArray(50000 * 24), DeviceArray(200000 * 4)
    cap = 3 * 12 ** 3 + 100  # room for three chunks' cases only
    d_cases = DeviceArray(cap + 4096)
    guard = np.full(cap + 4096, 0xAB, np.uint8)
    abi.check(abi.lib().uww_memcpy(ctx.h, C.c_void_p(d_cases.ptr), guard.ctypes.data_as(C.c_void_p), guard.size, 0))
    out = abi.MeshOut(d_v.ptr, None, d_i.ptr, d_cases.ptr, None, d_rec.ptr, d_tot.ptr, 50000, 200000, cap, 0)
    assert abi.lib().uww_build_chunks(ctx.h, C.c_void_p(d_desc.ptr), 8, 12, C.byref(out)) == abi.UWW_OK
    ctx.sync()
    tot = ctx.download(d_tot, (4,), np.uint64)
    assert int(tot[3]) & abi.UWW_ERRFLAG_RANGE
    back = ctx.download(d_cases, (cap + 4096,), np.uint8)
    assert np.all(back[cap:] == 0xAB), "nothing written past the capacity"


def test_fast_build_against_f64_oracle(ctx_factory, oracle):
    """The FMA build: count flipped cells and the worst vertex error vs the f64 oracle."""
    p, d = workloads.uniform_grid(seed=0, outputs=abi.UWW_OUT_CASES)
    sel = relayout(d[(d["pos"][:, 0] < 8) & (d["pos"][:, 1] < 8)])
    ref = oracle.build_chunks(p, sel, precision=oracle.F64)
    q = p.copy()
    q.math_mode = abi.UWW_MATH_FAST
    got = ctx_factory(q).build_chunks_device(sel, int(ref.totals[0]) + 4096, int(ref.totals[1]) + 16384)
    exact = ctx_factory(p).build_chunks_device(sel, int(ref.totals[0]) + 4096, int(ref.totals[1]) + 16384)
    assert got.status == abi.UWW_OK and exact.status == abi.UWW_OK

    def vertex_error(b):
        same = b.records["num_inds"] == ref.records["num_inds"]
        errs = []
        for i in np.nonzero(same & (ref.records["num_inds"] > 0))[0]:
            gv, _, gi = b.chunk(i)
            rv, _, ri = ref.chunk(i)
            if np.array_equal(gi, ri):
                errs.append(np.abs(gv["pos"] - rv["pos"]).max(axis=1))
        e = np.concatenate(errs)
        return float(e.max()), float(np.median(e))

    flips_fast = flipped_cells(got.cases, ref.cases)
    flips_exact = flipped_cells(exact.cases, ref.cases)
    fast_max, fast_med = vertex_error(got)
    exact_max, exact_med = vertex_error(exact)
    print(f"vs f64 oracle over {len(ref.cases)} cells: fast build {flips_fast} flipped cells, max vertex error "
          f"{fast_max:.3g} (median {fast_med:.3g}); exact f32 build {flips_exact} flipped, max {exact_max:.3g} "
          f"(median {exact_med:.3g}) world units")
    assert flips_fast <= 1e-4 * len(ref.cases), flips_fast
    # f32 noise against f64 noise: errors concentrate on near-degenerate edges
    # (both endpoint samples close to the iso-level); bound them at 1% of a cell
    cell = 16.0 / 12
    assert fast_max < 0.01 * cell and exact_max < 0.01 * cell, (fast_max, exact_max)
    assert fast_med < 1e-4 and exact_med < 1e-4


def test_fast_build_colours_and_normals_against_the_oracle(ctx_factory, oracle):
    """The fast build's pass 2 (hardware powf and quotient, FMA-contracted
    analytic gradient) against the F32 oracle's colours and normals, at the
    vertices of every chunk whose index buffer matches the oracle's; the
    bounds are written here: colours 2e-5 (a fraction of one 8-bit step),
    normals 2e-4 for 99.9 % of the vertices and 5e-3 for all (vertices on
    nearly degenerate edges move, and their normal with them; measured on
    GB300: colour 7.6e-6, normal p99.9 5.7e-5, max 6.5e-4)."""
    p, d = workloads.uniform_grid(seed=0, outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS)
    sel = relayout(d[(d["pos"][:, 0] < 8) & (d["pos"][:, 1] < 8)])
    ref = oracle.build_chunks(p, sel, precision=oracle.F32)
    q = p.copy()
    q.math_mode = abi.UWW_MATH_FAST
    got = ctx_factory(q).build_chunks_device(sel, int(ref.totals[0]) + 4096, int(ref.totals[1]) + 16384)
    assert got.status == abi.UWW_OK
    col_err, nrm_err = [], []
    for i in np.nonzero((got.records["num_inds"] == ref.records["num_inds"]) & (ref.records["num_inds"] > 0))[0]:
        gv, gn, gi = got.chunk(i)
        rv, rn, ri = ref.chunk(i)
        if not np.array_equal(gi, ri):
            continue
        col_err.append(np.abs(gv["color"] - rv["color"]).max(axis=1))
        nrm_err.append(np.abs(gn - rn).max(axis=1))
    col_err, nrm_err = np.concatenate(col_err), np.concatenate(nrm_err)
    print(f"fast pass 2 vs F32 oracle over {len(nrm_err)} vertices: colour max {col_err.max():.3g}, "
          f"normal max {nrm_err.max():.3g}, p99.9 {np.percentile(nrm_err, 99.9):.3g}, median {np.median(nrm_err):.3g}")
    assert len(nrm_err) > 10000
    assert col_err.max() < 2e-5, col_err.max()
    assert np.percentile(nrm_err, 99.9) < 2e-4 and nrm_err.max() < 5e-3, (np.percentile(nrm_err, 99.9), nrm_err.max())


@pytest.mark.parametrize("which", ["reference", "mixed", "lod24"])
def test_fast_build_other_workloads(ctx_factory, oracle, which):
    """The fast (column) noise on the terraced reference world, mixed LODs and 24^3 chunks."""
    if which == "reference":
        p, d = workloads.reference_grid(outputs=abi.UWW_OUT_CASES)
    elif which == "mixed":
        p, d = workloads.mixed_lod(seed=1, outputs=abi.UWW_OUT_CASES)
        d = relayout(d[:128])
    else:
        p, d = workloads.uniform_grid(seed=2, outputs=abi.UWW_OUT_CASES)
        d = make_descs(d["pos"][(d["pos"][:, 2] >= 6) & (d["pos"][:, 2] <= 9)][:64], 24)
    ref = oracle.build_chunks(p, d, precision=oracle.F64)
    q = p.copy()
    q.math_mode = abi.UWW_MATH_FAST
    got = ctx_factory(q).build_chunks_device(d, int(ref.totals[0]) + 8192, int(ref.totals[1]) + 32768)
    assert got.status == abi.UWW_OK
    flips = flipped_cells(got.cases, ref.cases)
    print(f"{which}: {flips} flipped of {len(ref.cases)} cells")
    assert flips <= max(2, 1e-4 * len(ref.cases)), flips
    blank_ref = (ref.records["flags"] & abi.UWW_CHUNK_HAS_MESH) > 0
    blank_got = (got.records["flags"] & abi.UWW_CHUNK_HAS_MESH) > 0
    assert np.count_nonzero(blank_ref != blank_got) <= 1


@pytest.mark.parametrize("shift", [0, 4, 8, 12, 1])
def test_host_build_into_page_locked_buffers(ctx_factory, shift):
    """uww_build_chunks_host with page-locked (device-addressable) buffers:
    records, indices, vertices and normals are streamed to the host during
    the build, cases by one copy kernel, with one synchronisation; the result
    is the device build's.  `shift` moves every output buffer off a 16-byte
    boundary by that many bytes (single-word stores; off a 4-byte boundary,
    the sized-copy path)."""
    import ctypes as C
    from underwaterworld_gb300.chunk import HostArray
    p, d = workloads.uniform_grid(seed=4, outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS | abi.UWW_OUT_CASES)
    p.math_mode = abi.UWW_MATH_FAST
    d = relayout(d[::5])
    ctx = ctx_factory(p)
    want = ctx.build_chunks_device(d, 1 << 20, 1 << 22)
    n, nc = len(d), int((d["cells"].astype(np.int64) ** 3).sum())
    vcap, icap = int(want.totals[0]) + 7, int(want.totals[1]) + 5   # odd sizes: unaligned tails
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
    pc, hc = host((nc,), np.uint8)
    tot = np.zeros(4, np.uint64)
    hd = HostArray((n,), abi.CHUNK_DESC_DTYPE)
    hd.array[:] = d
    out = abi.MeshOut(pv, pn, pi, pc, None, pr, tot.ctypes.data, vcap, icap, nc, 0)
    abi.check(abi.lib().uww_build_chunks_host(ctx.h, C.c_void_p(hd.ptr), n, C.byref(out)))
    nv, ni = int(tot[0]), int(tot[1])
    np.testing.assert_array_equal(tot[:3], want.totals[:3])
    np.testing.assert_array_equal(hr, want.records)
    np.testing.assert_array_equal(hv[:nv], want.verts)
    np.testing.assert_array_equal(hn[:nv], want.normals)
    np.testing.assert_array_equal(hi[:ni], want.inds)
    np.testing.assert_array_equal(hc, want.cases)


def test_host_build_streamed_positions_only(ctx_factory, oracle):
    """Streamed host output with neither colours nor normals requested: pass 2
    still runs to move the positions to the host; parity build bit-exact."""
    import ctypes as C
    from underwaterworld_gb300.chunk import HostArray
    p, d = workloads.reference_grid(outputs=0)
    ctx = ctx_factory(p)
    ref = oracle.build_chunks(p, d)
    vcap, icap = caps(ref)
    n = len(d)
    hv = HostArray((vcap,), abi.VERT_COLOR_DTYPE)
    hi = HostArray((icap,), np.uint32)
    hr = HostArray((n,), abi.CHUNK_RECORD_DTYPE)
    hd = HostArray((n,), abi.CHUNK_DESC_DTYPE)
    hd.array[:] = d
    tot = np.zeros(4, np.uint64)
    out = abi.MeshOut(hv.ptr, None, hi.ptr, None, None, hr.ptr, tot.ctypes.data, vcap, icap)
    abi.check(abi.lib().uww_build_chunks_host(ctx.h, C.c_void_p(hd.ptr), n, C.byref(out)))
    nv, ni = int(tot[0]), int(tot[1])
    assert (nv, ni) == (int(ref.totals[0]), int(ref.totals[1]))
    assert_records_equal(hr.array, ref.records)
    np.testing.assert_array_equal(hi.array[:ni], ref.inds)
    np.testing.assert_array_equal(hv.array[:nv]["pos"], ref.verts["pos"])
    assert not hv.array[:nv]["color"].any()


def test_misaligned_device_outputs_are_refused(ctx_factory):
    """Device outputs off the alignment the kernels store with (8 bytes for
    vertices and totals, 4 for the rest) and descriptors off a 4-byte
    boundary are refused on the host, before any launch."""
    import ctypes as C
    import torch
    p, d = workloads.reference_grid()
    ctx = ctx_factory(p)
    dev = torch.device("cuda")
    n = len(d)
    dd = torch.zeros(n * 32 + 16, dtype=torch.uint8, device=dev)
    dd[:n * 32] = torch.from_numpy(d.view(np.uint8).copy()).to(dev)
    bufs = {k: torch.zeros(1 << 20, dtype=torch.uint8, device=dev) for k in ("v", "n", "i", "r", "t")}
    base = {k: b.data_ptr() for k, b in bufs.items()}
    L = abi.lib()

    def run(desc_ptr, **shift):
        ptr = {k: base[k] + shift.get(k, 0) for k in base}
        out = abi.MeshOut(ptr["v"], ptr["n"], ptr["i"], None, None, ptr["r"], ptr["t"], 1 << 14, 1 << 16)
        return L.uww_build_chunks(ctx.h, C.c_void_p(desc_ptr), n, 12, C.byref(out))

    for shift in ({"v": 4}, {"t": 4}, {"i": 2}, {"n": 1}, {"r": 2}):
        assert run(dd.data_ptr(), **shift) == abi.UWW_ERR_INVALID_ARG, shift
    assert run(dd.data_ptr() + 2) == abi.UWW_ERR_INVALID_ARG
    assert run(dd.data_ptr()) == abi.UWW_OK
    torch.cuda.synchronize()


def test_surface_layer_bit_exact(ctx_factory, oracle):
    """A layer of 1024 chunks on the surface, nearly all meshed: the batched
    build's look-back, emission and vertex pass under a dense work queue."""
    p = workloads.fbm_params(5, 4, 0.04, -0.03, 128.0, 0.0, ALL)
    g = np.arange(32)
    pos = np.stack(np.meshgrid(g, g, [8], indexing="ij"), -1).reshape(-1, 3)
    d = make_descs(pos, 12)
    ref = oracle.build_chunks(p, d)
    meshed = int((ref.records["flags"] & abi.UWW_CHUNK_HAS_MESH).astype(bool).sum())
    assert meshed > 900, meshed
    got = ctx_factory(p).build_chunks_device(d, *caps(ref))
    assert_batches_equal(got, ref)


def test_dense_meshes_bit_exact(ctx_factory, oracle):
    """Dense meshes (high frequency, no depth bias): thousands of triangles
    per chunk, emitted a triangle per thread over many rounds."""
    p = workloads.fbm_params(6, 2, 0.3, 0.0, 0.0, 0.0, ALL)
    g = np.arange(8)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    d = make_descs(pos, 12)
    ref = oracle.build_chunks(p, d)
    tris = ref.records["num_inds"].astype(np.int64) // 3
    assert tris.min() > 3000, tris.min()
    got = ctx_factory(p).build_chunks_device(d, *caps(ref))
    assert_batches_equal(got, ref)


@pytest.mark.parametrize("bias", ["terraced", "linear"])
def test_depth_bias_bound_decides_far_chunks(ctx_factory, oracle, bias):
    """Chunks far above or below the surface are decided by the depth bias
    and the fBm bound without their noise: a tall column of chunks crossing
    the cut-off on both sides, bit-exact against the oracle (records, cases,
    mesh), and the samples output (which disables the shortcut) unchanged."""
    if bias == "terraced":
        p = abi.reference_params()
        p.outputs = ALL
        zs = np.arange(-12, 13)
    else:
        p = workloads.fbm_params(7, 4, 0.04, -0.03, 128.0, 0.0, ALL)
        zs = np.arange(0, 16)
    g = np.arange(2)
    pos = np.stack(np.meshgrid(g, g, zs, indexing="ij"), -1).reshape(-1, 3)
    d = make_descs(pos, 12)
    ref = oracle.build_chunks(p, d)
    flags = ref.records["flags"]
    assert (flags & abi.UWW_CHUNK_EARLY_BLANK).any() and (flags & abi.UWW_CHUNK_HAS_MESH).any()
    got = ctx_factory(p).build_chunks_device(d, *caps(ref))
    assert_batches_equal(got, ref)
    assert (got.cases.reshape(len(d), -1) == 255).all(axis=1).any()  # solid chunks
    q = p.copy()
    q.outputs = ALL | abi.UWW_OUT_SAMPLES
    with_samples = ctx_factory(q).build_chunks_device(d, *caps(ref))
    assert_batches_equal(with_samples, ref)
    want = np.concatenate([oracle.sample_grid(q, d[i]) for i in range(len(d))])
    np.testing.assert_array_equal(with_samples.samples, want)


def test_depth_shortcut_off_gives_the_same_output(ctx_factory, oracle):
    """UWW_TUNE_NO_DEPTH_SHORTCUT evaluates the noise of every chunk, also of
    those the depth bias decides; the output is the same bit for bit."""
    p, d = workloads.uniform_grid(seed=1, outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS)
    ref = oracle.build_chunks(p, d)
    ctx = ctx_factory(p)
    on = ctx.build_chunks_device(d, *caps(ref))
    ctx.set_tuning(options=abi.UWW_TUNE_NO_DEPTH_SHORTCUT)
    off = ctx.build_chunks_device(d, *caps(ref))
    ctx.set_tuning(options=0)
    assert_batches_equal(off, ref)
    assert_batches_equal(on, off)
    np.testing.assert_array_equal(on.verts, off.verts)
    np.testing.assert_array_equal(on.normals, off.normals)


def test_long_runs_of_bias_decided_chunks(ctx_factory, oracle):
    """A tall column of chunks, nearly all far above or below the surface:
    control warps run through long runs of depth-bias-decided tickets, more
    than a CTA keeps pending (their records then resolved at once).  Records,
    mesh and totals equal the oracle's."""
    p = abi.reference_params()
    p.outputs = abi.UWW_OUT_COLOR
    g = np.arange(2)
    pos = np.stack(np.meshgrid(g, g, np.arange(-1500, 1500), indexing="ij"), -1).reshape(-1, 3)
    d = make_descs(pos, 12)
    ref = oracle.build_chunks(p, d)
    assert (ref.records["flags"] & abi.UWW_CHUNK_HAS_MESH).sum() > 0
    ctx = ctx_factory(p)
    ctx.set_tuning(threads=192, blocks_per_sm=1)  # 152 CTAs: ~79 tickets each, most decided
    got = ctx.build_chunks_device(d, *caps(ref))
    assert got.status == abi.UWW_OK
    assert_batches_equal(got, ref)
    np.testing.assert_array_equal(got.totals[:3], ref.totals[:3])
