"""Queries against built chunks: per-cell triangle offsets (Chunk::tris_around,
chunk.rs:315-342) and the boids' wall-avoidance rays (boid.rs:175-244 with
util::Tri::intersects, util.rs:23-58), against the CPU restatement on the same
mesh.  Hit distances are compared bit for bit (f32, no FMA on either side)."""
import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import make_descs
from underwaterworld_gb300.query import WALL_RANGE, RayScene

pytestmark = pytest.mark.gpu


def unit(v):
    v = np.asarray(v, np.float32)
    n = np.sqrt((v * v).sum(-1, keepdims=True, dtype=np.float32)).astype(np.float32)
    return (v / n).astype(np.float32)


@pytest.fixture(scope="module")
def scene_and_oracle(built_lib):
    from oracle import oracle as O
    from underwaterworld_gb300.chunk import Context
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_CASES)
    p.math_mode = abi.UWW_MATH_EXACT
    ctx = Context(p)
    sc = RayScene(ctx, d)
    yield p, d, sc, O
    ctx.close()


def test_cell_tri_offsets_match_the_oracle(scene_and_oracle):
    p, d, sc, O = scene_and_oracle
    b = sc.batch()
    np.testing.assert_array_equal(sc.cell_first(), O.cell_tri_offsets(d, b.cases))


@pytest.mark.parametrize("rng", [WALL_RANGE, 6])
def test_ray_hits_match_the_oracle(scene_and_oracle, rng):
    p, d, sc, O = scene_and_oracle
    b = sc.batch()
    r = np.random.default_rng(rng)
    # boids near the surface (around mesh vertices) and anywhere in the grid
    near = b.verts["pos"][r.integers(0, len(b.verts), 300)] + r.normal(0, 1.5, (300, 3)).astype(np.float32)
    far = r.uniform(-36, 44, (100, 3)).astype(np.float32)
    origins = np.concatenate([near, far]).astype(np.float32)
    dirs = unit(r.normal(size=(len(origins), 18, 3)))
    got = sc.cast(origins, dirs, rng)
    want = O.ray_query(p, d, b, origins, dirs, rng)
    assert (want >= 0).sum() > 200, "the sample should hit walls"
    np.testing.assert_array_equal(got, want)


def test_boid_decisions_follow(scene_and_oracle):
    """heading_for_collision / safe_dir of boid.rs:209-244 from the nearest hits."""
    p, d, sc, O = scene_and_oracle
    b = sc.batch()
    r = np.random.default_rng(9)
    origins = b.verts["pos"][r.integers(0, len(b.verts), 64)] + r.normal(0, 1.0, (64, 3)).astype(np.float32)
    dirs = unit(r.normal(size=(64, 18, 3)))
    t = sc.cast(origins, dirs)
    heading = ((t[:, :2] >= 0) & (t[:, :2] < WALL_RANGE)).any(1)
    safe = ~((t[:, 2:] >= 0) & (t[:, 2:] <= WALL_RANGE))
    want = O.ray_query(p, d, b, origins, dirs, WALL_RANGE)
    np.testing.assert_array_equal(heading, ((want[:, :2] >= 0) & (want[:, :2] < WALL_RANGE)).any(1))
    np.testing.assert_array_equal(safe, ~((want[:, 2:] >= 0) & (want[:, 2:] <= WALL_RANGE)))
    assert heading.any()


def test_missing_chunks_and_empty_queries(built_lib):
    from underwaterworld_gb300.chunk import Context
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_CASES)
    with Context(p) as ctx:
        sub = make_descs(d["pos"][d["pos"][:, 0] <= 0], 12)   # only half the grid is built
        sc = RayScene(ctx, sub)
        t = sc.cast(np.array([[40.0, 0.0, 0.0], [-5.0, 3.0, 1.0]], np.float32), unit(np.ones((2, 4, 3))))
        assert np.all(t[0] == -1)          # no chunk there
        assert t.shape == (2, 4)
