"""The CPU oracle against the known-answer fixtures and its own invariants."""
import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.chunk import make_descs

from helpers import COLOR_ATOL, load_golden, params_for_samples


@pytest.mark.parametrize("name", ["single_cell", "single_cell_random", "grids"])
def test_oracle_matches_known_answers(oracle, name):
    g = load_golden(name)
    p = params_for_samples(g["iso_level"])
    b = oracle.build_chunks(p, g["descs"], samples_in=g["samples"])
    np.testing.assert_array_equal(b.records["num_verts"], g["num_verts"])
    np.testing.assert_array_equal(b.records["num_inds"], g["num_inds"])
    np.testing.assert_array_equal(b.inds, g["inds"])
    np.testing.assert_array_equal(b.cases, g["cases"])
    np.testing.assert_array_equal(b.verts["pos"], g["verts"])
    np.testing.assert_allclose(b.verts["color"], g["colors"], rtol=0, atol=COLOR_ATOL)


def test_single_cell_midpoints(oracle):
    """+-1 corner samples at iso 0: every vertex is an edge midpoint."""
    g = load_golden("single_cell")
    p = params_for_samples(0.0)
    b = oracle.build_chunks(p, g["descs"], samples_in=g["samples"])
    frac = np.modf(b.verts["pos"] / (16.0 / 1.0))[0]
    assert np.all(np.isin(np.round(np.abs(frac) * 2, 6), [0.0, 1.0]))


def test_perm_is_a_permutation_and_matches_product(oracle, built_lib):
    for seed in [0, 1, 2, 9, 12345, 2**31 - 1, 2**32 - 1]:
        pr = oracle.perm(seed)
        assert sorted(pr) == list(range(256))
        assert pr == abi.perm_table(seed), seed
    assert oracle.perm(0) != oracle.perm(1)


def test_perlin_lattice_zero_and_range(oracle):
    pts = np.stack(np.meshgrid(*[np.arange(-3, 4)] * 3, indexing="ij"), -1).reshape(-1, 3).astype(float)
    assert np.all(oracle.perlin(0, pts) == 0.0)  # gradient noise vanishes on the lattice
    rng = np.random.default_rng(1)
    v = oracle.perlin(0, rng.uniform(-100, 100, (20000, 3)))
    assert np.abs(v).max() < 1.2 and 0.1 < np.abs(v).mean() < 0.5


def test_perlin_f32_close_to_f64(oracle):
    rng = np.random.default_rng(2)
    pts = rng.uniform(-20, 20, (5000, 3)).astype(np.float32).astype(float)
    a = oracle.perlin(3, pts, precision=oracle.F64)
    b = oracle.perlin(3, pts, precision=oracle.F32)
    assert np.abs(a - b).max() < 2e-5


def test_density_gradient_matches_finite_differences(oracle):
    p, _ = workloads.uniform_grid(seed=1)
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 256, (200, 3)).astype(np.float32)
    _, g = oracle.density_at(p, x, precision=oracle.F64, grad=True)
    h = 1e-2
    fd = np.zeros_like(g, dtype=np.float64)
    for ax in range(3):
        e = np.zeros(3, np.float32)
        e[ax] = h
        fd[:, ax] = (oracle.density_at(p, x + e, precision=oracle.F64).astype(np.float64)
                     - oracle.density_at(p, x - e, precision=oracle.F64).astype(np.float64)) / (2 * h)
    np.testing.assert_allclose(g, fd, atol=2e-3)


def test_linear_and_hashed_dedup_agree(oracle):
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_CASES)
    a = oracle.build_chunks(p, d, precision=oracle.F64, search=oracle.SEARCH_LINEAR)
    b = oracle.build_chunks(p, d, precision=oracle.F64, search=oracle.SEARCH_HASHED)
    np.testing.assert_array_equal(a.inds, b.inds)
    np.testing.assert_array_equal(a.verts, b.verts)


def test_threads_do_not_change_results(oracle):
    p, d = workloads.reference_grid()
    a = oracle.build_chunks(p, d, threads=1)
    b = oracle.build_chunks(p, d, threads=4)
    np.testing.assert_array_equal(a.records, b.records)
    np.testing.assert_array_equal(a.inds, b.inds)
    np.testing.assert_array_equal(a.verts, b.verts)


def test_reference_grid_structure(oracle):
    """The 5x5x5 reference grid at the reference iso-level: blank chunks, u16-sized meshes, terraced surface."""
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_CASES)
    b = oracle.build_chunks(p, d, precision=oracle.F64)
    r = b.records
    early = (r["flags"] & abi.UWW_CHUNK_EARLY_BLANK) > 0
    mesh = (r["flags"] & abi.UWW_CHUNK_HAS_MESH) > 0
    assert early.sum() > 0 and mesh.sum() > 0
    assert not np.any(early & mesh)
    assert np.all((r["num_inds"] > 0) == mesh)
    assert np.all(r["num_inds"] % 3 == 0)
    assert int(r["num_verts"].max()) < 65536  # the reference's u16 index buffers hold
    for i in np.nonzero(mesh)[0][:10]:
        inds = b.inds[r["ind_offset"][i]:r["ind_offset"][i] + r["num_inds"][i]]
        assert inds.max() == r["num_verts"][i] - 1
        # vertex ids appear in first-use order
        first = np.unique(inds, return_index=True)[1]
        assert np.all(np.diff(inds[np.sort(first)]) == 1)


def test_edge_dedup_has_fewer_vertices(oracle):
    p, d = workloads.reference_grid()
    a = oracle.build_chunks(p, d)
    p.dedup_mode = abi.UWW_DEDUP_EDGE
    b = oracle.build_chunks(p, d)
    assert int(b.totals[0]) < int(a.totals[0])
    assert int(b.totals[1]) == int(a.totals[1])


def test_capacity_overflow_reports_counts(oracle):
    p, d = workloads.reference_grid()
    full = oracle.build_chunks(p, d)
    small = oracle.build_chunks(p, d, vert_capacity=100, ind_capacity=100)
    assert small.status == abi.UWW_ERR_CAPACITY
    np.testing.assert_array_equal(small.totals[:2], full.totals[:2])
    assert int(small.totals[2]) > 0


def test_empty_batch(oracle):
    p = abi.reference_params()
    b = oracle.build_chunks(p, make_descs(np.zeros((0, 3)), 12))
    assert b.totals[0] == 0 and b.totals[1] == 0 and len(b.records) == 0


def test_oracle_range_checks_per_cell_outputs(oracle):
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_CASES)
    sub = d[[0, 5, 9]]  # offsets still those of the full grid: beyond a 3-chunk buffer
    with pytest.raises(RuntimeError):
        oracle.build_chunks(p, sub)


def test_perlin_bound_used_by_the_depth_bias_shortcut():
    """The build decides a chunk from its depth bias when the bias keeps every
    sample beyond the iso level by more than the fBm can reach, with
    |Perlin| <= 1.11 before the 2/sqrt(3) output scale.  The bound: per corner
    |g . d| <= S = |dx|+|dy|+|dz| - min(...) for gradients with two +-1
    components, F = sum_c W_c S_c on a 201^3 grid, plus the Lipschitz margin
    |grad F| <= 8.5 sqrt(3) times the largest distance to a grid point."""
    def fade(t):
        return t * t * t * (t * (t * 6 - 15) + 10)
    n = 201
    u = np.linspace(0.0, 1.0, n)
    U, V, W = np.meshgrid(u, u, u, indexing="ij")
    F = np.zeros_like(U)
    for cx in (0, 1):
        for cy in (0, 1):
            for cz in (0, 1):
                w = (fade(U) if cx else 1 - fade(U)) * (fade(V) if cy else 1 - fade(V)) * \
                    (fade(W) if cz else 1 - fade(W))
                dx, dy, dz = np.abs(U - cx), np.abs(V - cy), np.abs(W - cz)
                F += w * (dx + dy + dz - np.minimum(np.minimum(dx, dy), dz))
    h = 1.0 / (n - 1)
    bound = F.max() + 8.5 * np.sqrt(3) * h * np.sqrt(3) / 2
    assert F.max() < 1.037 and bound <= 1.11, (F.max(), bound)
    # the oracle's Perlin (scaled by 2/sqrt(3)) stays inside the bound
    from oracle import oracle as O
    rng = np.random.default_rng(0)
    xyz = rng.uniform(-300, 300, (200_000, 3))
    for seed in (0, 1, 7):
        v = O.perlin(seed, xyz)
        assert np.abs(v).max() <= 1.0364 * 2 / np.sqrt(3) + 1e-9, np.abs(v).max()


def test_depth_bias_decided_chunks_have_no_mesh_in_the_oracle(oracle):
    """The chunks bench.py counts as decided by the depth bias (its float32
    restatement of the build's test, which sets the roofline's flop count) are,
    in the oracle at both precisions, early blank (every sample above the iso
    level) or solid (every case 255): none of them has a mesh."""
    import bench
    from underwaterworld_gb300 import abi
    from underwaterworld_gb300.chunk import make_descs
    p, d = bench.workload(3)
    p.outputs = abi.UWW_OUT_CASES
    mask = bench.bias_decided_mask(p, d)
    assert mask.sum() == 2560
    sub = d[mask][::8]
    sub = make_descs(sub["pos"], sub["cells"])
    for prec in (oracle.F32, oracle.F64):
        b = oracle.build_chunks(p, sub, precision=prec)
        assert (b.records["num_inds"] == 0).all()
        blank = (b.records["flags"] & abi.UWW_CHUNK_EARLY_BLANK) != 0
        solid = (b.cases.reshape(len(sub), -1) == 255).all(axis=1)
        assert (blank | solid).all()
        assert blank.any() and solid.any()
