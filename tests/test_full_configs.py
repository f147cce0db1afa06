"""Parity on the benchmark's full workloads, not subsets.

* The uniform grid the headline times -- 16x16x16 = 4096 chunks of 12^3
  cells, 4-octave fBm minus 0.03 (z - 128), iso-level 0 -- for every
  permutation seed 0-9 the benchmark cycles through, built by the parity
  build (UWW_MATH_EXACT) and compared with the F32 oracle: records (counts,
  offsets, flags), index buffers and vertex positions bit-exact, colours
  within COLOR_ATOL, normals within NORMAL_ATOL.  Twice per seed: with the
  benchmark's outputs (colour + normals, so the control warps settle the
  chunks the depth bias decides) and with per-cell cases as well (every chunk
  through the compute warps, cases compared bit for bit).
* The whole 2048-chunk uneven-LOD batch (12^3 / 24^3 / 48^3 at 50/35/15 %,
  6-octave fBm), the same comparison.
* The fast build (UWW_MATH_FAST) on the whole uniform grid against the F64
  oracle (the reference's f64 noise): flipped cells and vertex error,
  bounded.
* The two batched builds -- the split build (front kernel, then emission of
  every triangle; the default for these 12^3 chunks) and the single
  pipelined kernel (UWW_TUNE_PIPELINED) -- give the same bytes on the whole
  uniform grid, fast build with the benchmark's outputs.

The oracle follows chunk.rs:105-264 and perlin_util.rs:6-29.
"""
import os

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads

from helpers import assert_batches_equal

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
COLOR_NORMALS = abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS
ALL = COLOR_NORMALS | abi.UWW_OUT_CASES


def caps(ref):
    return max(int(ref.totals[0]), 1), max(int(ref.totals[1]), 1)


@pytest.mark.parametrize("seed", range(10))
def test_uniform_grid_every_chunk_every_seed_bit_exact(ctx_factory, oracle, seed):
    for outputs in (COLOR_NORMALS, ALL):
        p, d = workloads.uniform_grid(seed=seed, outputs=outputs)
        assert len(d) == 4096
        ref = oracle.build_chunks(p, d, precision=oracle.F32, threads=THREADS)
        got = ctx_factory(p).build_chunks_device(d, *caps(ref))
        assert got.status == abi.UWW_OK
        assert_batches_equal(got, ref)
        assert (ref.records["flags"] & abi.UWW_CHUNK_HAS_MESH).sum() > 1000


def test_mixed_lod_whole_batch_bit_exact(ctx_factory, oracle):
    p, d = workloads.mixed_lod(seed=0, outputs=ALL)
    assert len(d) == 2048 and set(np.unique(d["cells"])) == {12, 24, 48}
    ref = oracle.build_chunks(p, d, precision=oracle.F32, threads=THREADS)
    got = ctx_factory(p).build_chunks_device(d, *caps(ref))
    assert got.status == abi.UWW_OK
    assert_batches_equal(got, ref)


def test_fast_build_whole_grid_against_f64_oracle(ctx_factory, oracle):
    """Every seed of the headline grid, fast build vs the f64 oracle."""
    rows = []
    for seed in range(10):
        p, d = workloads.uniform_grid(seed=seed, outputs=abi.UWW_OUT_CASES)
        ref = oracle.build_chunks(p, d, precision=oracle.F64, threads=THREADS)
        q = p.copy()
        q.math_mode = abi.UWW_MATH_FAST
        got = ctx_factory(q).build_chunks_device(d, int(ref.totals[0]) + 4096, int(ref.totals[1]) + 16384)
        assert got.status == abi.UWW_OK
        rows.append(oracle.fast_vs_reference(got, ref))
    cells = sum(r["cells"] for r in rows)
    flips = sum(r["flipped_cells"] for r in rows)
    worst = max(r["max_vertex_err"] for r in rows)
    print(f"fast build vs f64 oracle, 10 seeds x 4096 chunks: {flips} flipped of {cells} cells, "
          f"max vertex error {worst:.3g} world units")
    assert flips <= 1e-5 * cells, flips
    assert worst < 0.01 * 16.0 / 12, worst  # 1 % of a cell
    assert max(r["median_vertex_err"] for r in rows) < 1e-4


@pytest.mark.parametrize("seed", [0, 3, 7])
def test_split_and_pipelined_builds_give_the_same_bytes(ctx_factory, seed):
    p, d = workloads.uniform_grid(seed=seed, outputs=COLOR_NORMALS)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = ctx_factory(p)
    split = ctx.build_chunks_device(d, 400_000, 1_500_000)
    ctx.set_tuning(options=abi.UWW_TUNE_PIPELINED)
    piped = ctx.build_chunks_device(d, 400_000, 1_500_000)
    ctx.set_tuning(options=0)
    again = ctx.build_chunks_device(d, 400_000, 1_500_000)
    for b in (split, piped, again):
        assert b.status == abi.UWW_OK
    assert (split.records["flags"] & abi.UWW_CHUNK_HAS_MESH).sum() > 1000
    for other in (piped, again):
        np.testing.assert_array_equal(split.records, other.records)
        np.testing.assert_array_equal(split.totals, other.totals)
        np.testing.assert_array_equal(split.inds, other.inds)
        np.testing.assert_array_equal(split.verts.view(np.uint32), other.verts.view(np.uint32))
        np.testing.assert_array_equal(split.normals.view(np.uint32), other.normals.view(np.uint32))
