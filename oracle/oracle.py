"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, to verify libuww_gb300.so against.  The product
never imports this module.  See uww_oracle.c for what it restates and the
parity status of each part.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

# struct layouts only: importing them never loads the GPU library
from underwaterworld_gb300 import layout
from underwaterworld_gb300.layout import MeshBatch, total_cells, total_samples

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

F32, F64 = 0, 1
SEARCH_LINEAR, SEARCH_HASHED = 0, 1

_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        L.oracle_perm.argtypes = [C.c_uint32, P]
        L.oracle_perm.restype = None
        L.oracle_build_chunks.argtypes = [C.POINTER(layout.Params), C.c_int, C.c_int, P, C.c_uint32,
                                          C.POINTER(layout.MeshOut), C.c_int, P, C.c_uint64]
        L.oracle_build_chunks.restype = C.c_int
        L.oracle_sample_grid.argtypes = [C.POINTER(layout.Params), C.c_int, P, P]
        L.oracle_sample_grid.restype = C.c_int
        L.oracle_density_at.argtypes = [C.POINTER(layout.Params), C.c_int, P, C.c_uint32, P, P]
        L.oracle_density_at.restype = C.c_int
        L.oracle_perlin.argtypes = [C.c_uint32, C.c_int, P, C.c_uint32, P]
        L.oracle_perlin.restype = C.c_int
        L.oracle_adjoint64.argtypes = [C.POINTER(layout.Params), P, P, C.c_uint32, P, P, P, P, P, P, P, P, P, P]
        L.oracle_adjoint64.restype = C.c_int
        L.oracle_cell_tri_offsets.argtypes = [P, C.c_uint32, P, P]
        L.oracle_cell_tri_offsets.restype = C.c_int
        L.oracle_ray_query.argtypes = [C.POINTER(layout.Params), P, C.c_uint32, P, P, P, P, P, C.c_uint32, P,
                                       C.c_uint32, C.c_int32, P]
        L.oracle_ray_query.restype = C.c_int
        L.oracle_schedule_chunks.argtypes = [C.POINTER(layout.Params), C.POINTER(layout.ScheduleParams), P, P, C.c_uint32,
                                             P, C.c_uint32, P, C.c_uint32, P]
        L.oracle_schedule_chunks.restype = C.c_int
        L.oracle_shade_vertices.argtypes = [C.POINTER(layout.CameraUniform), P, C.c_uint32, P, P, P]
        L.oracle_shade_vertices.restype = C.c_int
        _lib = L
    return _lib


def perm(seed: int) -> bytes:
    buf = (C.c_uint8 * 256)()
    lib().oracle_perm(seed, buf)
    return bytes(buf)


def build_chunks(params: layout.Params, descs: np.ndarray, precision: int = F32, search: int = SEARCH_HASHED,
                 threads: int = 1, samples_in: np.ndarray | None = None, vert_capacity: int | None = None,
                 ind_capacity: int | None = None) -> MeshBatch:
    descs = np.ascontiguousarray(descs, dtype=layout.CHUNK_DESC_DTYPE)
    n = descs.shape[0]
    nc, ns = total_cells(descs), total_samples(descs)
    vcap = vert_capacity if vert_capacity is not None else 15 * nc
    icap = ind_capacity if ind_capacity is not None else 15 * nc
    records = np.zeros(n, dtype=layout.CHUNK_RECORD_DTYPE)
    verts = np.empty(vcap, dtype=layout.VERT_COLOR_DTYPE)
    normals = np.empty((vcap, 3), dtype=np.float32) if params.outputs & layout.UWW_OUT_NORMALS else None
    inds = np.empty(icap, dtype=np.uint32)
    cases = np.zeros(nc, dtype=np.uint8) if params.outputs & layout.UWW_OUT_CASES else None
    samples = np.zeros(ns, dtype=np.float32) if params.outputs & layout.UWW_OUT_SAMPLES else None
    totals = np.zeros(4, dtype=np.uint64)

    def ptr(a):
        return a.ctypes.data if a is not None else None

    out = layout.MeshOut(ptr(verts), ptr(normals), ptr(inds), ptr(cases), ptr(samples), ptr(records), ptr(totals),
                      vcap, icap, cases.size if cases is not None else 0, samples.size if samples is not None else 0)
    sin = np.ascontiguousarray(samples_in, dtype=np.float32) if samples_in is not None else None
    st = lib().oracle_build_chunks(C.byref(params), precision, search, descs.ctypes.data_as(C.c_void_p), n,
                                   C.byref(out), threads, ptr(sin), sin.size if sin is not None else 0)
    if st not in (layout.UWW_OK, layout.UWW_ERR_CAPACITY):
        raise RuntimeError(f"oracle_build_chunks failed: {st}")
    nv, ni = min(int(totals[0]), vcap), min(int(totals[1]), icap)
    return MeshBatch(records, verts[:nv].copy(), normals[:nv].copy() if normals is not None else None,
                     inds[:ni].copy(), cases, totals, st, samples)


def sample_grid(params: layout.Params, desc, precision: int = F32) -> np.ndarray:
    d = np.ascontiguousarray(np.asarray(desc, dtype=layout.CHUNK_DESC_DTYPE).reshape(1))
    S = int(d["cells"][0]) + 1
    out = np.zeros(S ** 3, dtype=np.float32)
    st = lib().oracle_sample_grid(C.byref(params), precision, d.ctypes.data_as(C.c_void_p),
                                  out.ctypes.data_as(C.c_void_p))
    if st:
        raise RuntimeError(f"oracle_sample_grid failed: {st}")
    return out


def density_at(params: layout.Params, xyz: np.ndarray, precision: int = F32, grad: bool = False):
    xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
    n = xyz.shape[0]
    out = np.zeros(n, dtype=np.float32)
    g = np.zeros((n, 3), dtype=np.float32) if grad else None
    st = lib().oracle_density_at(C.byref(params), precision, xyz.ctypes.data_as(C.c_void_p), n,
                                 out.ctypes.data_as(C.c_void_p), g.ctypes.data_as(C.c_void_p) if grad else None)
    if st:
        raise RuntimeError(f"oracle_density_at failed: {st}")
    return (out, g) if grad else out


def perlin(seed: int, xyz: np.ndarray, precision: int = F64) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(xyz.shape[0], dtype=np.float64)
    lib().oracle_perlin(seed, precision, xyz.ctypes.data_as(C.c_void_p), xyz.shape[0],
                        out.ctypes.data_as(C.c_void_p))
    return out


# ---- topology-frozen adjoint (FP64 reference) ---------------------------------
def theta_of(params: layout.Params) -> np.ndarray:
    """theta = (effective per-octave amplitudes, base_freq, offset xyz, iso) in f64."""
    K = int(params.octaves)
    amps, a = [], np.float32(params.amplitude)
    for k in range(K):
        amps.append(float(params.amps[k]) if params.explicit_amps else float(a))
        a = np.float32(a * np.float32(params.persistence))
    return np.array(amps + [params.base_freq, *params.offset, params.iso_level], dtype=np.float64)


def adjoint64(params: layout.Params, descs: np.ndarray, records: np.ndarray, edge_ids: np.ndarray,
              pos_grad: np.ndarray, theta: np.ndarray | None = None, samples_in: np.ndarray | None = None,
              want_theta: bool = True, want_samples: bool = False, want_positions: bool = False,
              want_dmax: bool = False, want_pole: bool = False) -> dict:
    """FP64 loss sum_v pos_grad[v] . p_v over the given edges, and its gradients."""
    descs = np.ascontiguousarray(descs, dtype=layout.CHUNK_DESC_DTYPE)
    records = np.ascontiguousarray(records, dtype=layout.CHUNK_RECORD_DTYPE)
    edge_ids = np.ascontiguousarray(edge_ids, dtype=np.uint32)
    pos_grad = np.ascontiguousarray(pos_grad, dtype=np.float32).reshape(-1, 3)
    K = int(params.octaves)
    th = np.ascontiguousarray(theta, dtype=np.float64) if theta is not None else None
    sin = np.ascontiguousarray(samples_in, dtype=np.float64) if samples_in is not None else None
    loss = C.c_double()
    tg = np.zeros(K + 5) if want_theta else None
    sg = np.zeros(total_samples(descs)) if want_samples else None
    pos = np.zeros((edge_ids.size, 3)) if want_positions else None
    dmax = np.zeros(K + 5) if want_dmax else None
    pole = np.zeros(K + 5) if want_pole else None

    def ptr(a):
        return a.ctypes.data if a is not None else None

    st = lib().oracle_adjoint64(C.byref(params), ptr(th), descs.ctypes.data, descs.shape[0], records.ctypes.data,
                                edge_ids.ctypes.data, pos_grad.ctypes.data, ptr(sin), C.byref(loss), ptr(tg),
                                ptr(sg), ptr(pos), ptr(dmax), ptr(pole))
    if st:
        raise RuntimeError(f"oracle_adjoint64 failed: {st}")
    return {"loss": loss.value, "theta_grad": tg, "sample_grad": sg, "positions": pos, "dmax": dmax, "pole": pole}


def fd_theta(params: layout.Params, descs, records, edge_ids, pos_grad, h: float = 1e-4, theta=None,
             richardson: bool = False, pole_frac: float = 0.02) -> tuple:
    """FP64 central differences of the loss in theta.  The step of parameter i
    is h in units of its effect on the density: h / max|d rho/d theta_i| over
    the samples the vertices use (so no sample moves by more than h; for the
    iso level and amplitudes that is about h itself), and at most pole_frac of
    the distance in theta_i to the nearest degenerate edge (where t has a
    pole: the loss is rational in each theta_i, and a stencil wider than the
    pole distance differentiates across the pole).  With richardson, the
    central differences at h and h/2 are combined to cancel the h^2 error term.
    Returns (fd, steps)."""
    th = theta_of(params) if theta is None else np.asarray(theta, np.float64)
    r = adjoint64(params, descs, records, edge_ids, pos_grad, theta=th, want_theta=False, want_dmax=True,
                  want_pole=True)
    steps = np.minimum(h / np.maximum(r["dmax"], 1.0), pole_frac * r["pole"])

    def central(i, s):
        tp, tm = th.copy(), th.copy()
        tp[i] += s
        tm[i] -= s
        lp = adjoint64(params, descs, records, edge_ids, pos_grad, theta=tp, want_theta=False)["loss"]
        lm = adjoint64(params, descs, records, edge_ids, pos_grad, theta=tm, want_theta=False)["loss"]
        return (lp - lm) / (2 * s)

    fd = np.zeros_like(th)
    for i in range(th.size):
        fd[i] = central(i, steps[i])
        if richardson:  # (4 D(h/2) - D(h)) / 3 cancels the h^2 term
            fd[i] = (4 * central(i, steps[i] / 2) - fd[i]) / 3
    return fd, steps


def crossing_edges(params: layout.Params, descs: np.ndarray, samples: np.ndarray):
    """Every grid edge whose two samples lie on opposite sides of the iso-level
    (one vertex per edge), as records + edge ids in the forward's encoding:
    id = (sample index << 3) | dir, from the lower sample in direction +axis."""
    descs = np.ascontiguousarray(descs, dtype=layout.CHUNK_DESC_DTYPE)
    iso = np.float32(params.iso_level)
    recs = np.zeros(descs.shape[0], dtype=layout.CHUNK_RECORD_DTYPE)
    ids, off = [], 0
    for i, d in enumerate(descs):
        S = int(d["cells"]) + 1
        rho = samples[int(d["sample_offset"]):int(d["sample_offset"]) + S ** 3].reshape(S, S, S)
        inside = rho < iso
        idx = np.arange(S ** 3, dtype=np.uint32).reshape(S, S, S)
        mine = []
        for axis in range(3):
            lo = [slice(None)] * 3
            hi = [slice(None)] * 3
            lo[axis] = slice(0, S - 1)
            hi[axis] = slice(1, S)
            cross = inside[tuple(lo)] != inside[tuple(hi)]
            mine.append((idx[tuple(lo)][cross] << 3) | np.uint32(2 * axis))
        e = np.concatenate(mine).astype(np.uint32)
        recs[i]["num_verts"] = e.size
        recs[i]["vert_offset"] = off
        recs[i]["flags"] = layout.UWW_CHUNK_HAS_MESH if e.size else 0
        ids.append(e)
        off += e.size
    return recs, (np.concatenate(ids) if ids else np.zeros(0, np.uint32))


# ---- queries against built chunks ------------------------------------------------
def cell_tri_offsets(descs: np.ndarray, cases: np.ndarray) -> np.ndarray:
    descs = np.ascontiguousarray(descs, dtype=layout.CHUNK_DESC_DTYPE)
    cases = np.ascontiguousarray(cases, dtype=np.uint8)
    first = np.zeros(cases.size, np.uint32)
    lib().oracle_cell_tri_offsets(descs.ctypes.data, descs.shape[0], cases.ctypes.data, first.ctypes.data)
    return first


def ray_query(params: layout.Params, descs, batch: MeshBatch, origins: np.ndarray, dirs: np.ndarray, rng: int):
    """Nearest hit per (query, ray) against the triangles around each query point."""
    descs = np.ascontiguousarray(descs, dtype=layout.CHUNK_DESC_DTYPE)
    origins = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
    nq = origins.shape[0]
    dirs = np.ascontiguousarray(dirs, dtype=np.float32).reshape(nq, -1, 3)
    nr = dirs.shape[1]
    out = np.zeros((nq, nr), np.float32)
    recs = np.ascontiguousarray(batch.records)
    verts = np.ascontiguousarray(batch.verts)
    inds = np.ascontiguousarray(batch.inds)
    cases = np.ascontiguousarray(batch.cases)
    st = lib().oracle_ray_query(C.byref(params), descs.ctypes.data, descs.shape[0], recs.ctypes.data, verts.ctypes.data,
                                inds.ctypes.data, cases.ctypes.data, origins.ctypes.data, nq, dirs.ctypes.data, nr,
                                rng, out.ctypes.data)
    if st:
        raise RuntimeError(f"oracle_ray_query failed: {st}")
    return out


def schedule_chunks(params: layout.Params, sp, known_descs=None, known_records=None, cap: int = 4096):
    """World::update_nearby: (generation list descriptors in GenPrio order, render list (m, 3))."""
    n_known = 0 if known_descs is None else len(known_descs)
    kd = np.ascontiguousarray(known_descs if n_known else np.zeros(1, layout.CHUNK_DESC_DTYPE), dtype=layout.CHUNK_DESC_DTYPE)
    kr = np.ascontiguousarray(known_records if n_known else np.zeros(1, layout.CHUNK_RECORD_DTYPE),
                              dtype=layout.CHUNK_RECORD_DTYPE)
    gen = np.zeros(cap, layout.CHUNK_DESC_DTYPE)
    ren = np.zeros((cap, 3), np.int32)
    counts = np.zeros(2, np.uint32)
    st = lib().oracle_schedule_chunks(C.byref(params), C.byref(sp), kd.ctypes.data, kr.ctypes.data, n_known,
                                      gen.ctypes.data, cap, ren.ctypes.data, cap, counts.ctypes.data)
    if st:
        raise RuntimeError(f"oracle_schedule_chunks failed: {st}")
    return gen[:counts[0]], ren[:counts[1]]


def shade_vertices(cam, verts: np.ndarray):
    """terrain.wgsl at each vertex: (clip (V, 4), rgb (V, 3), dist_light (V, 2))."""
    verts = np.ascontiguousarray(verts, dtype=layout.VERT_COLOR_DTYPE)
    nv = verts.shape[0]
    clip, rgb, dl = np.zeros((nv, 4), np.float32), np.zeros((nv, 3), np.float32), np.zeros((nv, 2), np.float32)
    lib().oracle_shade_vertices(C.byref(cam), verts.ctypes.data, nv, clip.ctypes.data, rgb.ctypes.data, dl.ctypes.data)
    return clip, rgb, dl


# ---- accuracy of a GPU build against an oracle build of the same chunks -----------
def fast_vs_reference(got: MeshBatch, ref: MeshBatch) -> dict:
    """Flipped cells (case indices that differ; both builds need per-cell cases)
    and the vertex position error over the chunks whose index buffers are
    identical (same topology, so vertices correspond one to one), in world
    units: max and median over vertices of the largest coordinate error."""
    flipped = int(np.count_nonzero(got.cases != ref.cases))
    errs = []
    same = got.records["num_inds"] == ref.records["num_inds"]
    compared = 0
    for i in np.nonzero(same & (ref.records["num_inds"] > 0))[0]:
        gv, _, gi = got.chunk(i)
        rv, _, ri = ref.chunk(i)
        if np.array_equal(gi, ri):
            errs.append(np.abs(gv["pos"].astype(np.float64) - rv["pos"].astype(np.float64)).max(axis=1))
            compared += 1
    e = np.concatenate(errs) if errs else np.zeros(1)
    meshed = int((ref.records["num_inds"] > 0).sum())
    return {"cells": int(ref.cases.size), "flipped_cells": flipped, "max_vertex_err": float(e.max()),
            "median_vertex_err": float(np.median(e)), "vertices_compared": int(e.size if errs else 0),
            "meshed_chunks": meshed, "chunks_same_topology": compared}
