"""uww_build_chunks_noalloc: the batched build for callers that cannot allocate.

Callers such as an engine whose allocator owns all device memory, or a frame
callback that must not call cudaMalloc, build chunks into buffers they already
own through this entry point; its scratch is a fixed array inside the library.
This file checks, through the C ABI, that two calls in a row give exactly the
output of the allocating entry point (uww_build_chunks) for the same inputs.
Every buffer here is allocated by the test (as such a caller's allocator
would) before the calls under test.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import Context, DeviceArray, make_descs

pytestmark = pytest.mark.gpu

OUTPUTS = abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS | abi.UWW_OUT_CASES


class Buffers:
    """Caller-owned device buffers for one build of `n` chunks."""

    def __init__(self, n, ncells, vcap, icap):
        self.vcap, self.icap, self.n, self.ncells = vcap, icap, n, ncells
        self.verts = DeviceArray(vcap * 24)
        self.normals = DeviceArray(vcap * 12)
        self.inds = DeviceArray(icap * 4)
        self.cases = DeviceArray(ncells)
        self.records = DeviceArray(n * 32)
        self.totals = DeviceArray(32)

    def out(self):
        return abi.MeshOut(self.verts.ptr, self.normals.ptr, self.inds.ptr, self.cases.ptr, None, self.records.ptr,
                           self.totals.ptr, self.vcap, self.icap, self.ncells, 0)

    def fetch(self, ctx):
        tot = ctx.download(self.totals, (4,), np.uint64)
        nv, ni = int(tot[0]), int(tot[1])
        return {
            "totals": tot,
            "records": ctx.download(self.records, (self.n,), abi.CHUNK_RECORD_DTYPE),
            "verts": ctx.download(self.verts, (nv,), abi.VERT_COLOR_DTYPE),
            "normals": ctx.download(self.normals, (nv, 3), np.float32),
            "inds": ctx.download(self.inds, (ni,), np.uint32),
            "cases": ctx.download(self.cases, (self.ncells,), np.uint8),
        }


def assert_same(a, b):
    np.testing.assert_array_equal(a["totals"], b["totals"])
    np.testing.assert_array_equal(a["records"], b["records"])
    np.testing.assert_array_equal(a["inds"], b["inds"])
    np.testing.assert_array_equal(a["cases"], b["cases"])
    np.testing.assert_array_equal(a["verts"]["pos"], b["verts"]["pos"])
    # same kernel, same inputs: colours and normals agree to the tolerances of
    # the other parity tests (they are in fact identical)
    np.testing.assert_allclose(a["verts"]["color"], b["verts"]["color"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(a["normals"], b["normals"], rtol=0, atol=1e-6)


@pytest.mark.parametrize("math_mode", [abi.UWW_MATH_EXACT, abi.UWW_MATH_FAST])
def test_noalloc_matches_allocating_build_twice(math_mode):
    p, d = workloads.uniform_grid(seed=7, outputs=OUTPUTS)
    p.math_mode = math_mode
    sel = d[(d["pos"][:, 0] < 8) & (d["pos"][:, 1] < 8)]
    descs = make_descs(sel["pos"], sel["cells"])
    n, ncells = len(descs), int((descs["cells"].astype(np.int64) ** 3).sum())
    vcap, icap = 400_000, 1_200_000

    with Context(p) as ctx:
        d_desc = ctx.upload(descs)
        ref_buf = Buffers(n, ncells, vcap, icap)
        ref_out = ref_buf.out()
        abi.check(abi.lib().uww_build_chunks(ctx.h, C.c_void_p(d_desc.ptr), n, 12, C.byref(ref_out)), "reference build")
        ctx.sync()
        ref = ref_buf.fetch(ctx)
        assert int(ref["totals"][2]) == 0 and int(ref["totals"][3]) == 0
        assert int(ref["totals"][1]) > 0

        # two calls in a row into fresh caller-owned buffers, on the context's stream
        for _ in range(2):
            buf = Buffers(n, ncells, vcap, icap)
            out = buf.out()
            st = abi.lib().uww_build_chunks_noalloc(C.byref(p), C.c_void_p(ctx.stream()), C.c_void_p(d_desc.ptr), n,
                                                    12, C.byref(out))
            abi.check(st, "uww_build_chunks_noalloc")
            ctx.sync()
            assert_same(buf.fetch(ctx), ref)


def test_noalloc_smaller_batch_after_a_larger_one():
    """The array keeps the last call's contents: a call with fewer chunks
    after a larger one still starts from cleared scratch and gives the
    allocating build's output."""
    p, d = workloads.uniform_grid(seed=9, outputs=OUTPUTS)
    p.math_mode = abi.UWW_MATH_FAST
    big = make_descs(d["pos"][:2048], d["cells"][:2048])
    small = make_descs(d["pos"][1500:1564], d["cells"][1500:1564])
    vcap, icap = 300_000, 1_000_000
    with Context(p) as ctx:
        results = []
        for descs in (big, small):
            n, ncells = len(descs), int((descs["cells"].astype(np.int64) ** 3).sum())
            d_desc = ctx.upload(descs)
            ref_buf, buf = Buffers(n, ncells, vcap, icap), Buffers(n, ncells, vcap, icap)
            ref_out, out = ref_buf.out(), buf.out()
            abi.check(abi.lib().uww_build_chunks(ctx.h, C.c_void_p(d_desc.ptr), n, 12, C.byref(ref_out)))
            abi.check(abi.lib().uww_build_chunks_noalloc(C.byref(p), C.c_void_p(ctx.stream()), C.c_void_p(d_desc.ptr),
                                                         n, 12, C.byref(out)))
            ctx.sync()
            results.append((buf.fetch(ctx), ref_buf.fetch(ctx)))
        for got, ref in results:
            assert int(ref["totals"][2]) == 0 and int(ref["totals"][3]) == 0
            assert_same(got, ref)
        assert int(results[1][1]["totals"][1]) > 0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    p, d = workloads.uniform_grid(seed=1)
    with Context(p) as ctx:
        d_desc = ctx.upload(d[:4])
        buf = Buffers(4, 4 * 12 ** 3, 1000, 1000)
        out = buf.out()
        L = abi.lib()
        # more chunks than the fixed scratch holds
        assert L.uww_build_chunks_noalloc(C.byref(p), C.c_void_p(ctx.stream()), C.c_void_p(d_desc.ptr), 65537, 12,
                                          C.byref(out)) == abi.UWW_ERR_INVALID_ARG
        # chunks whose working set would need a global scratch slot
        assert L.uww_build_chunks_noalloc(C.byref(p), C.c_void_p(ctx.stream()), C.c_void_p(d_desc.ptr), 4, 48,
                                          C.byref(out)) == abi.UWW_ERR_INVALID_ARG
        # no totals: a timeout, bad descriptor or overflow could not be reported
        out.totals = None
        assert L.uww_build_chunks_noalloc(C.byref(p), C.c_void_p(ctx.stream()), C.c_void_p(d_desc.ptr), 4, 12,
                                          C.byref(out)) == abi.UWW_ERR_INVALID_ARG
