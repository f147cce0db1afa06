"""Sizing of the split build's slabs (uww_internal.h, host side; no GPU).

A chunk of 17..63 cells per edge is built as slabs of K x layers, one CTA of
kSlabThreads threads each.  The kernels rely on these facts about K, for
every N:
  * the slab's (K+1) x planes of sample columns fit one pass of the CTA's
    threads (one column per thread in the column noise);
  * its workspace fits the budget, and with the z tables and column masks the
    split build's dynamic shared memory stays under the per-CTA limit;
  * its cell index fits the 16 bits it has in an active-cell list entry;
  * its vertices fit 16-bit ids in both dedup modes (slab_vertex_bound), and
    that bound is the count a slab reaches when every edge is crossed: checked
    here by counting the (corner a, corner b) keys of a 3D checkerboard in the
    reference's corner order (chunk.rs:144-153, marching_table.rs:1-14), at
    sizes where the count takes a moment;
  * the slabs cover the chunk, the last one possibly shorter.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SMEM_PER_CTA = 227 * 1024

# corner offsets (x, y, z) and edge -> (corner a, corner b), reference order
CORNER = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]
EDGE = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


@pytest.fixture(scope="module")
def sizes(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path_factory.mktemp("slab") / "slab_sizes"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "--expt-relaxed-constexpr",
           f"-I{ROOT / 'include'}", f"-I{ROOT / 'underwaterworld_gb300' / 'csrc'}",
           str(HERE / "cpp" / "slab_sizes.cu"), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    lines = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    threads, budget, act_cap, max_cells, chunk16 = map(int, lines[0].split())
    rows = [tuple(map(int, ln.split())) for ln in lines[1:] if ln.strip()]
    return dict(threads=threads, budget=budget, act_cap=act_cap, max_cells=max_cells, chunk16=chunk16, rows=rows)


def max_first_slab_vertices(N, K, oriented):
    """Distinct vertex keys created by the first slab (x layers 0..K-1) of an
    N-cell chunk whose every edge is crossed."""
    keys = set()
    for x in range(K):
        for y in range(N):
            for z in range(N):
                for a, b in EDGE:
                    pa = (x + CORNER[a][0], y + CORNER[a][1], z + CORNER[a][2])
                    pb = (x + CORNER[b][0], y + CORNER[b][1], z + CORNER[b][2])
                    keys.add((pa, pb) if oriented else (min(pa, pb), max(pa, pb)))
    return len(keys)


def vertex_bound(N, K):
    S = N + 1
    return max(K * S * S + 2 * (K + 1) * N * S, (5 * K + 1) * N * S)


@pytest.mark.parametrize("N,K", [(3, 2), (5, 1), (6, 4), (9, 3)])
def test_vertex_bound_is_the_checkerboard_count(N, K):
    S = N + 1
    assert max_first_slab_vertices(N, K, True) == (5 * K + 1) * N * S
    assert max_first_slab_vertices(N, K, False) == K * S * S + 2 * (K + 1) * N * S


def test_every_slab_size_fits_its_limits(sizes):
    assert sizes["max_cells"] == 63 and len(sizes["rows"]) == 63 - 17 + 1
    ws_max = sizes["chunk16"]
    for N, K, count, ws, vbound, ztab in sizes["rows"]:
        S = N + 1
        assert 1 <= K <= N
        assert (K + 1) * S <= sizes["threads"], N
        assert ws <= sizes["budget"], N
        # a batch of up to N cells: the largest workspace so far, the fast
        # build's z tables (16 octaves) and a 16^3 chunk's column masks
        ws_max = max(ws_max, ws)
        dyn = ((ws_max + ztab + 15) & ~15) + 13 * 13 * 8
        assert dyn <= SMEM_PER_CTA, N
        assert K * N * N < 1 << 16, N
        assert vbound == vertex_bound(N, K) and vbound < 1 << 16, N
        assert count == -(-N // K) and (count - 1) * K < N <= count * K, N
        # a staged reference into the previous slab: bit 31, the owner's edge
        # in bits 24..27, its cell's y * N + z below them
        assert N * N < 1 << 24, N
        # queue entry: chunk | slab << 24
        assert count < 1 << 8, N
    # an active-cell list entry: the cell's first triangle in 16 bits (at most
    # 5 triangles a cell, and the list holds act_cap cells)
    assert 5 * sizes["act_cap"] < 1 << 16
