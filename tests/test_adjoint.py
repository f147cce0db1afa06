"""Topology-frozen adjoint: uww_forward / uww_backward / uww_height_loss.

CPU tests pin the FP64 oracle gradient against FP64 central finite
differences; GPU tests compare the library's f32 forward and backward with
that oracle on the same edges.  Tolerances:
  * dL/dtheta vs FP64 finite differences and vs the FP64 CPU gradient:
    1e-4 relative (per entry, against max(|entry|, 1e-3 * max |gradient|));
  * dL/d(sample): 1e-4 relative to the largest entry;
  * positions rebuilt from the edge ids in f64: 2e-5 world units (f32 rounding
    of coordinates up to ~200).
"""
import ctypes as C

import numpy as np
import pytest

from underwaterworld_gb300 import abi, workloads
from underwaterworld_gb300.adjoint import (Adjoint, TerrainFit, gaussian_heightmap, params_with_theta,
                                           terrain_volume, theta_from_params)
from underwaterworld_gb300.chunk import DeviceArray, make_descs

GRAD_RTOL = 1e-4


def rel_err(got, want):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    floor = 1e-3 * np.abs(want).max()
    return np.abs(got - want) / np.maximum(np.abs(want), floor)


def small_case(oracle, normalize=1, bias=None, cells=12):
    p, d = workloads.uniform_grid(seed=5, outputs=abi.UWW_OUT_SAMPLES)
    p.normalize = normalize
    if bias == "terraced":
        p.bias_mode, p.bias_a, p.bias_b, p.bias_c = abi.UWW_BIAS_TERRACED, 16.0, 32.0, 0.25
        p.base_freq = 1.0 / 16.0
        pos = np.array([[x, y, z] for x in range(-1, 2) for y in range(-1, 2) for z in range(-1, 2)])
    else:
        pos = np.array([[x, y, z] for x in range(2) for y in range(2) for z in range(7, 10)])
    descs = make_descs(pos, np.full(len(pos), cells))
    b = oracle.build_chunks(p, descs, precision=oracle.F32)
    recs, eids = oracle.crossing_edges(p, descs, b.samples)
    c = workloads.cotangents(recs, eids, seed=1)
    return p, descs, recs, eids, c, b.samples


# ---- CPU: the FP64 oracle gradient against FP64 finite differences ---------------
@pytest.mark.parametrize("normalize,bias", [(1, None), (0, None), (1, "terraced")])
def test_oracle_theta_gradient_matches_finite_differences(oracle, normalize, bias):
    p, descs, recs, eids, c, _ = small_case(oracle, normalize, bias)
    assert eids.size > 500
    r = oracle.adjoint64(p, descs, recs, eids, c)
    fd, steps = oracle.fd_theta(p, descs, recs, eids, c, h=1e-4, richardson=True)
    assert np.all(steps <= 1e-4)
    err = rel_err(r["theta_grad"], fd)
    if bias == "terraced":
        # The terrace adj - fmod(adj, 0.25), adj = (z + offset_z) * f / 2, is a step
        # function; the reference grid puts samples exactly on its steps
        # (world z = 8m), where d/df and d/doffset_z do not exist and central
        # differences straddle the jump.  The adjoint uses the step's derivative
        # 0; the other entries must still match.
        K = int(p.octaves)
        err = np.delete(err, [K, K + 3])
    assert err.max() < 1e-6, (err, r["theta_grad"], fd)


def test_oracle_sample_gradient_matches_finite_differences(oracle):
    p, descs, recs, eids, c, samples = small_case(oracle)
    s64 = samples.astype(np.float64)
    r = oracle.adjoint64(p, descs, recs, eids, c, samples_in=s64, want_samples=True, want_theta=True)
    # the iso-level derivative is the only theta entry with samples given
    assert np.all(r["theta_grad"][:-1] == 0) and r["theta_grad"][-1] != 0
    g = r["sample_grad"]
    rng = np.random.default_rng(0)
    touched = np.flatnonzero(g)
    pick = np.concatenate([rng.choice(touched, 40, replace=False), rng.choice(np.flatnonzero(g == 0), 5)])
    h = 1e-6
    for i in pick:
        sp, sm = s64.copy(), s64.copy()
        sp[i] += h
        sm[i] -= h
        lp = oracle.adjoint64(p, descs, recs, eids, c, samples_in=sp, want_theta=False)["loss"]
        lm = oracle.adjoint64(p, descs, recs, eids, c, samples_in=sm, want_theta=False)["loss"]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_oracle_loss_is_linear_in_cotangents(oracle):
    p, descs, recs, eids, c, _ = small_case(oracle)
    a = oracle.adjoint64(p, descs, recs, eids, c)
    b = oracle.adjoint64(p, descs, recs, eids, 2 * c)
    assert b["loss"] == pytest.approx(2 * a["loss"], rel=1e-12)
    np.testing.assert_allclose(b["theta_grad"], 2 * a["theta_grad"], rtol=1e-12)


def test_theta_roundtrip_and_heightmap():
    p, _ = workloads.adjoint_batch()
    th = theta_from_params(p)
    assert th.size == abi.theta_count(4) == 9
    q = params_with_theta(p, th)
    np.testing.assert_array_equal(theta_from_params(q), th)
    hm = gaussian_heightmap(16, 32.0, seed=3)
    assert hm.shape == (16, 16) and np.all(hm >= 0)
    np.testing.assert_array_equal(hm, gaussian_heightmap(16, 32.0, seed=3))
    rec = np.zeros(1, abi.CHUNK_RECORD_DTYPE)
    rec["num_verts"] = 4
    c1 = workloads.cotangents(rec, np.arange(4, dtype=np.uint32), seed=0)
    c2 = workloads.cotangents(rec, np.arange(4, dtype=np.uint32), seed=0)
    np.testing.assert_array_equal(c1, c2)


# ---- GPU: the library against the oracle --------------------------------------------
def run_forward(ctx, descs, vcap=1 << 20, icap=1 << 22, sample_grad=False):
    a = Adjoint(ctx, descs, vcap, icap, sample_grad=sample_grad)
    a.forward()
    ctx.sync()
    return a, a.fetch_forward()


@pytest.mark.gpu
@pytest.mark.parametrize("dedup", [abi.UWW_DEDUP_EDGE, abi.UWW_DEDUP_ORIENTED])
def test_forward_edge_ids_rebuild_the_vertices(ctx_factory, oracle, dedup):
    p, descs = workloads.adjoint_batch(side=4)
    p.math_mode = abi.UWW_MATH_EXACT
    p.dedup_mode = dedup
    p.outputs = abi.UWW_OUT_CASES | abi.UWW_OUT_SAMPLES
    ctx = ctx_factory(p)
    a, f = run_forward(ctx, descs)
    nv = f["edge_ids"].size
    assert nv > 1000
    # the same build's samples: positions rebuilt in f64 from the edge ids
    samples = ctx.build_chunks_device(descs, 1 << 20, 1 << 22).samples
    c = np.zeros((nv, 3), np.float32)
    r = oracle.adjoint64(p, descs, f["records"], f["edge_ids"], c, samples_in=samples.astype(np.float64),
                         want_theta=False, want_positions=True)
    np.testing.assert_allclose(f["verts"]["pos"], r["positions"], rtol=0, atol=2e-5)
    if dedup == abi.UWW_DEDUP_EDGE:
        # one vertex per crossed grid edge: the same edge set as the samples give
        recs, eids = oracle.crossing_edges(p, descs, samples)
        for i in range(len(descs)):
            g = f["records"][i]
            mine = f["edge_ids"][g["vert_offset"]:g["vert_offset"] + g["num_verts"]]
            # canonical form: lower sample, + direction
            S = int(descs[i]["cells"]) + 1
            strides = np.array([S * S, S, 1], np.uint32)
            sa, dr = mine >> 3, mine & 7
            neg = (dr & 1) == 1
            lo = np.where(neg, sa - strides[dr >> 1], sa)
            canon = np.sort((lo << 3) | (dr & 6))
            o, n = int(recs[i]["vert_offset"]), int(recs[i]["num_verts"])
            np.testing.assert_array_equal(canon, np.sort(eids[o:o + n]), err_msg=f"chunk {i}")


@pytest.mark.gpu
@pytest.mark.parametrize("math_mode", [abi.UWW_MATH_EXACT, abi.UWW_MATH_FAST])
def test_backward_matches_fp64_gradient_and_finite_differences(ctx_factory, oracle, math_mode):
    """Config-4 adjoint check: 512 chunks of 24^3 cells, 4-octave fBm."""
    p, descs = workloads.adjoint_batch()
    p.math_mode = math_mode
    ctx = ctx_factory(p)
    a, f = run_forward(ctx, descs, vcap=1 << 21, icap=1 << 23, sample_grad=True)
    c = workloads.cotangents(f["records"], f["edge_ids"], seed=0)
    a.set_pos_grad(c)
    a.backward()
    g_gpu = a.theta_grad()
    sg_gpu = a.sample_grad()
    assert np.all(np.isfinite(g_gpu))
    r = oracle.adjoint64(p, descs, f["records"], f["edge_ids"], c, want_samples=True)
    fd, _ = oracle.fd_theta(p, descs, f["records"], f["edge_ids"], c, h=1e-4, richardson=True)
    assert rel_err(r["theta_grad"], fd).max() < 1e-6
    e_ref = rel_err(g_gpu, r["theta_grad"])
    e_fd = rel_err(g_gpu, fd)
    assert e_ref.max() < GRAD_RTOL, (e_ref, g_gpu, r["theta_grad"])
    assert e_fd.max() < GRAD_RTOL, (e_fd, g_gpu, fd)
    sref = r["sample_grad"]
    assert np.abs(sg_gpu - sref).max() <= GRAD_RTOL * np.abs(sref).max()


@pytest.mark.gpu
def test_backward_is_deterministic_and_poisoned_by_bad_edge_ids(ctx_factory):
    p, descs = workloads.adjoint_batch(side=4)
    ctx = ctx_factory(p)
    a, f = run_forward(ctx, descs)
    c = workloads.cotangents(f["records"], f["edge_ids"], seed=2)
    a.set_pos_grad(c)
    a.backward()
    g1 = a.theta_grad()
    a.backward()
    np.testing.assert_array_equal(a.theta_grad(), g1)
    # an edge id pointing outside its chunk: every entry becomes NaN
    bad = np.array([0xFFFFFFF8], np.uint32)
    k = int(np.flatnonzero(f["records"]["num_verts"])[0])
    off = int(f["records"][k]["vert_offset"])
    abi.check(abi.lib().uww_memcpy(ctx.h, C.c_void_p(a.d_edges.ptr + 4 * off), bad.ctypes.data_as(C.c_void_p), 4,
                                   abi.H2D))
    ctx.sync()
    a.backward()
    assert np.all(np.isnan(a.theta_grad()))


@pytest.mark.gpu
def test_height_loss_matches_numpy(ctx_factory):
    p, descs = terrain_volume(chunks_per_edge=4, cells=16)
    ctx = ctx_factory(p)
    a, f = run_forward(ctx, descs)
    verts = f["verts"]["pos"]
    cols, col = 4, 16.0
    target = gaussian_heightmap(cols, col, seed=1, base=20.0)
    d_t = ctx.upload(target)
    d_work, d_loss = DeviceArray(4 * cols * cols * 4), DeviceArray(4)
    abi.check(abi.lib().uww_height_loss(ctx.h, C.c_void_p(a.d_verts.ptr), C.c_void_p(a.d_tot.ptr), a.vcap, 0.0, 0.0,
                                        col, cols, cols, C.c_void_p(d_t.ptr), C.c_void_p(d_work.ptr),
                                        C.c_void_p(a.d_pos_grad.ptr), C.c_void_p(d_loss.ptr)))
    ctx.sync()
    loss = ctx.download(d_loss, (1,), np.float32)[0]
    pg = ctx.download(a.d_pos_grad, (verts.shape[0], 3), np.float32)
    cx = np.floor(verts[:, 0] / col).astype(int)
    cy = np.floor(verts[:, 1] / col).astype(int)
    ok = (cx >= 0) & (cx < cols) & (cy >= 0) & (cy < cols)
    cid = np.where(ok, cy * cols + cx, 0)
    sums = np.bincount(cid[ok], weights=verts[ok, 2].astype(np.float64), minlength=cols * cols)
    cnt = np.bincount(cid[ok], minlength=cols * cols)
    hit = cnt > 0
    mean = np.where(hit, sums / np.maximum(cnt, 1), 0)
    res = mean - target.ravel()
    want = (res[hit] ** 2).sum() / (cols * cols)
    assert loss == pytest.approx(want, rel=1e-4)
    gz = np.where(ok, 2 * res[cid] / np.maximum(cnt[cid], 1) / (cols * cols), 0)
    np.testing.assert_allclose(pg[:, 2], gz, rtol=1e-4, atol=1e-9)
    assert np.all(pg[:, :2] == 0)


@pytest.mark.gpu
def test_terrain_fit_reduces_the_loss(ctx_factory):
    p, descs = terrain_volume(chunks_per_edge=4, cells=16, octaves=4)
    ctx = ctx_factory(p)
    target = gaussian_heightmap(2, 32.0, n_bumps=2, seed=4, sigma=(10.0, 30.0), height=(5.0, 15.0), base=24.0)
    fit = TerrainFit(ctx, descs, target, 32.0, vert_capacity=1 << 20, ind_capacity=1 << 22, lr=2e-2)
    res = fit.run(30)
    assert np.all(np.isfinite(res["losses"]))
    assert min(res["losses"][-5:]) < 0.7 * res["losses"][0], res["losses"]


def test_terrain_fit_state_round_trips_through_a_checkpoint_file(tmp_path):
    """The fit's state (theta0, scales, phi, Adam moments and step count,
    learning rate) survives save/load unchanged.  No GPU: the state is set
    on an instance without a context."""
    fit = TerrainFit.__new__(TerrainFit)
    rng = np.random.default_rng(3)
    fit.theta0, fit.scale, fit.phi = rng.normal(size=13), rng.uniform(0.1, 2, 13), rng.normal(size=13)
    fit.m, fit.v, fit.t, fit.lr = rng.normal(size=13), rng.uniform(0, 1, 13), 17, 0.01
    path = tmp_path / "fit.npz"
    fit.save(path)
    other = TerrainFit.__new__(TerrainFit)
    other.theta0 = np.zeros(13)
    other.load(path)
    for k, v in fit.state_dict().items():
        np.testing.assert_array_equal(np.asarray(other.state_dict()[k]), np.asarray(v), err_msg=k)
    wrong = TerrainFit.__new__(TerrainFit)
    wrong.theta0 = np.zeros(9)
    with pytest.raises(ValueError):
        wrong.load(path)


@pytest.mark.gpu
def test_terrain_fit_resumes_from_a_checkpoint(ctx_factory, tmp_path):
    """Ten steps straight equal five steps, a checkpoint, and five more steps
    of a new fit loaded from it: forward, heightmap loss and backward are
    deterministic, so the losses and theta agree bit for bit."""
    p, descs = terrain_volume(chunks_per_edge=4, cells=16, octaves=4)
    target = gaussian_heightmap(2, 32.0, n_bumps=2, seed=4, sigma=(10.0, 30.0), height=(5.0, 15.0), base=24.0)
    kw = dict(vert_capacity=1 << 20, ind_capacity=1 << 22, lr=2e-2)
    straight = TerrainFit(ctx_factory(p.copy()), descs, target, 32.0, **kw).run(10)
    ck = tmp_path / "fit.npz"
    first = TerrainFit(ctx_factory(p.copy()), descs, target, 32.0, **kw)
    head = first.run(5, checkpoint=ck, every=5)
    resumed = TerrainFit(ctx_factory(p.copy()), descs, target, 32.0, **kw)
    resumed.load(ck)
    tail = resumed.run(5)
    assert head["losses"] + tail["losses"] == straight["losses"]
    np.testing.assert_array_equal(tail["theta"], straight["theta"])
    assert np.isfinite(tail["grad_norm"])
