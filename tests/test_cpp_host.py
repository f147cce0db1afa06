"""The C++ chunk interface (underwaterworld_gb300/host/uww_chunk.hpp): the
reference's Chunk / Perlin / iso_at / tris_around API over the C ABI.  A C++
program (tests/cpp/chunk_api_test.cpp) builds the reference grid through it;
its dump is compared with the CPU oracle: positions, indices and case-derived
triangles exactly, colours within the parity tolerance."""
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads

from helpers import COLOR_ATOL

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpp" / "chunk_api_test.cpp"


@pytest.fixture(scope="module")
def program(built_lib, tmp_path_factory):
    from underwaterworld_gb300 import build as B
    exe = tmp_path_factory.mktemp("cpp") / "chunk_api_test"
    return B.build_host_program(SRC, exe)


def test_host_interface_compiles_and_links(program):
    assert program.exists()


def test_host_interface_fails_loudly_without_a_gpu(program, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([str(program), str(tmp_path / "d.bin")], capture_output=True, text=True)
    assert r.returncode == 1 and "uww error" in r.stderr


def read_dump(path):
    b = path.read_bytes()
    off = 0

    def arr(dtype):
        nonlocal off
        n = struct.unpack_from("<Q", b, off)[0]
        off += 8
        a = np.frombuffer(b[off:off + n], dtype=dtype).copy()
        off += n
        return a

    n = struct.unpack_from("<Q", b, off)[0]
    off += 8
    chunks = []
    for _ in range(n):
        nb = b[off]
        off += 1
        chunks.append({"not_blank": bool(nb), "verts": arr(abi.VERT_COLOR_DTYPE), "inds": arr(np.uint32),
                       "inds_u16": arr(np.uint16), "tris": arr(np.float32)})
    pts = arr(np.float32).reshape(-1, 3)
    iso = arr(np.float32)
    return chunks, pts, iso


def tris_around(verts, inds, cases, p, rng, N=12):
    """chunk.rs:315-342 + util.rs:12-21 in numpy float32 (no fused operations)."""
    from underwaterworld_gb300.csrc_tables import CASE_NTRI
    first = np.concatenate([[0], np.cumsum(3 * CASE_NTRI[cases])[:-1]]).astype(np.int64)
    m = [int(np.floor(np.float32(v) * np.float32(N))) for v in p]
    lo = [max(v - rng, 0) for v in m]
    hi = [min(v + rng, N - 1) for v in m]
    out = []
    for x in range(lo[0], hi[0] + 1):
        for y in range(lo[1], hi[1] + 1):
            for z in range(lo[2], hi[2] + 1):
                c = (x * N + y) * N + z
                for j in range(CASE_NTRI[cases[c]]):
                    v = [verts["pos"][inds[first[c] + 3 * j + k]].astype(np.float32) for k in range(3)]
                    e1, e2 = v[1] - v[0], v[2] - v[0]
                    n = np.array([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                  e1[0] * e2[1] - e1[1] * e2[0]], np.float32)
                    mag = np.sqrt(np.float32(n[0] * n[0]) + np.float32(n[1] * n[1]) + np.float32(n[2] * n[2]),
                                  dtype=np.float32)
                    if mag != 0:
                        n = (n / mag).astype(np.float32)
                    out.append(np.concatenate([v[0], v[1], v[2], n]))
    return np.array(out, np.float32).reshape(-1, 12)


@pytest.mark.gpu
def test_host_interface_matches_the_oracle(program, oracle, tmp_path):
    dump = tmp_path / "dump.bin"
    r = subprocess.run([str(program), str(dump)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    chunks, pts, iso = read_dump(dump)
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_CASES)
    ref = oracle.build_chunks(p, d, precision=oracle.F32)
    assert len(chunks) == len(d)
    ntris = 0
    for i, c in enumerate(chunks):
        v, _, ind = ref.chunk(i)
        assert c["not_blank"] == (int(ref.records["num_inds"][i]) > 0)
        np.testing.assert_array_equal(c["verts"]["pos"], v["pos"])
        np.testing.assert_allclose(c["verts"]["color"], v["color"], rtol=0, atol=COLOR_ATOL)
        np.testing.assert_array_equal(c["inds"], ind)
        np.testing.assert_array_equal(c["inds_u16"], ind.astype(np.uint16))
        cases = ref.cases[int(d["cell_offset"][i]):int(d["cell_offset"][i]) + 12 ** 3]
        t = c["tris"]
        o = 0
        for lp in ((0.5, 0.5, 0.5), (0.1, 0.8, 0.3), (0.95, 0.05, 0.6)):
            k = int(t[o])
            o += 1
            got = t[o:o + 12 * k].reshape(k, 12)
            o += 12 * k
            if not c["not_blank"]:
                assert k == 0
                continue
            np.testing.assert_array_equal(got, tris_around(v, ind, cases, lp, 3))
            ntris += k
    assert ntris > 100
    want = oracle.density_at(p, pts * np.float32(16.0))
    np.testing.assert_array_equal(iso, want)
