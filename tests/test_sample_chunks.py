"""uww_sample_chunks: the density samples of a batch (Chunk::build_iso,
chunk.rs:105-129) without the mesher.  They must equal, bit for bit, the
samples the batched build computes in the same math mode (UWW_OUT_SAMPLES),
and in the parity build the f32 oracle's samples."""
import ctypes as C

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import DeviceArray, make_descs

from helpers import relayout

pytestmark = pytest.mark.gpu


def build_samples(ctx, descs):
    b = ctx.build_chunks_device(descs, 1 << 21, 1 << 23)
    assert b.status == abi.UWW_OK
    return b.samples


@pytest.mark.parametrize("math_mode", [abi.UWW_MATH_FAST, abi.UWW_MATH_EXACT])
@pytest.mark.parametrize("workload", ["uniform", "mixed", "lods"])
def test_samples_equal_the_builds_samples(ctx_factory, math_mode, workload):
    if workload == "uniform":
        p, d = workloads.uniform_grid(seed=3, outputs=abi.UWW_OUT_SAMPLES)
        d = relayout(d[::7])
    elif workload == "mixed":
        p, d = workloads.mixed_lod(seed=2, n=300, outputs=abi.UWW_OUT_SAMPLES)
    else:
        # every size class of the sampler: register columns (12, 16, 24 cells),
        # the column loop in shared memory (5, 20) and in global memory (40, 64)
        p = workloads.fbm_params(1, 6, 0.03, 0.02, 0.0, 0.0, abi.UWW_OUT_SAMPLES)
        cells = np.array([12, 16, 24, 5, 20, 40, 64, 1, 12, 24])
        pos = np.stack([np.arange(len(cells)), np.zeros(len(cells)), np.zeros(len(cells))], 1) - np.array([5, 0, 0])
        d = make_descs(pos, cells)
    p.math_mode = math_mode
    ctx = ctx_factory(p)
    got = ctx.sample_chunks(d)
    want = build_samples(ctx, d)
    np.testing.assert_array_equal(got, want)


def test_parity_samples_match_the_oracle(ctx_factory, oracle):
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_SAMPLES)
    p.math_mode = abi.UWW_MATH_EXACT
    ctx = ctx_factory(p)
    got = ctx.sample_chunks(d)
    want = oracle.build_chunks(p, d, precision=oracle.F32).samples
    np.testing.assert_array_equal(got, want)


def test_bad_descriptors_are_flagged_and_skipped(ctx_factory):
    p, d = workloads.uniform_grid(seed=0)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    d = relayout(d[:3])
    d["cells"][1] = 13          # above max_cells = 12
    d_desc = ctx.upload(d)
    buf = DeviceArray(3 * 13 ** 3 * 4)
    L = abi.lib()
    abi.check(L.uww_sample_chunks(ctx.h, C.c_void_p(d_desc.ptr), 3, 12, C.c_void_p(buf.ptr), 3 * 13 ** 3))
    flags = C.c_uint32()
    abi.check(L.uww_sample_status(ctx.h, C.byref(flags)))
    assert flags.value & abi.UWW_ERRFLAG_BAD
    # samples beyond the capacity: not written, flagged
    d2 = relayout(d[:1])
    d2["sample_offset"][0] = 100
    d_desc2 = ctx.upload(d2)
    abi.check(L.uww_sample_chunks(ctx.h, C.c_void_p(d_desc2.ptr), 1, 12, C.c_void_p(buf.ptr), 13 ** 3))
    abi.check(L.uww_sample_status(ctx.h, C.byref(flags)))
    assert flags.value & abi.UWW_ERRFLAG_RANGE


def test_global_scratch_classification_matches_sampled_build(ctx_factory):
    """Chunks above the shared-memory cut keep their samples in global scratch
    and are classified from per-column inside masks; the same chunks built
    from their sampled densities (classified from the samples) give the same
    mesh, cases and records bit for bit."""
    from helpers import assert_batches_equal
    p = workloads.fbm_params(4, 6, 0.03, 0.02, 0.0, 0.0,
                             abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS | abi.UWW_OUT_CASES)
    p.math_mode = abi.UWW_MATH_FAST
    cells = np.array([24, 48, 12, 40, 64, 5, 24, 48, 33, 63])
    pos = np.stack([np.arange(len(cells)) - 5, np.zeros(len(cells)), np.arange(len(cells)) % 2 - 1], 1)
    d = make_descs(pos, cells)
    ctx = ctx_factory(p)
    samples = ctx.sample_chunks(d)
    a = ctx.build_chunks_device(d, 1 << 21, 1 << 23)
    b = ctx.build_chunks_device(d, 1 << 21, 1 << 23, samples_in=samples)
    assert a.status == abi.UWW_OK and b.status == abi.UWW_OK
    assert (a.records["flags"] & abi.UWW_CHUNK_HAS_MESH).sum() >= 6
    assert_batches_equal(a, b)
