"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker of libuww_gb300.so.  The product
never imports this module.  See uww_oracle.c for what it restates and the
parity status of each part.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from underwaterworld_gb300 import abi
from underwaterworld_gb300.chunk import MeshBatch, total_cells, total_samples

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
        L.oracle_build_chunks.argtypes = [C.POINTER(abi.Params), C.c_int, C.c_int, P, C.c_uint32,
                                          C.POINTER(abi.MeshOut), C.c_int, P, C.c_uint64]
        L.oracle_build_chunks.restype = C.c_int
        L.oracle_sample_grid.argtypes = [C.POINTER(abi.Params), C.c_int, P, P]
        L.oracle_sample_grid.restype = C.c_int
        L.oracle_density_at.argtypes = [C.POINTER(abi.Params), C.c_int, P, C.c_uint32, P, P]
        L.oracle_density_at.restype = C.c_int
        L.oracle_perlin.argtypes = [C.c_uint32, C.c_int, P, C.c_uint32, P]
        L.oracle_perlin.restype = C.c_int
        _lib = L
    return _lib


def perm(seed: int) -> bytes:
    buf = (C.c_uint8 * 256)()
    lib().oracle_perm(seed, buf)
    return bytes(buf)


def build_chunks(params: abi.Params, descs: np.ndarray, precision: int = F32, search: int = SEARCH_HASHED,
                 threads: int = 1, samples_in: np.ndarray | None = None, vert_capacity: int | None = None,
                 ind_capacity: int | None = None) -> MeshBatch:
    descs = np.ascontiguousarray(descs, dtype=abi.CHUNK_DESC_DTYPE)
    n = descs.shape[0]
    nc, ns = total_cells(descs), total_samples(descs)
    vcap = vert_capacity if vert_capacity is not None else 15 * nc
    icap = ind_capacity if ind_capacity is not None else 15 * nc
    records = np.zeros(n, dtype=abi.CHUNK_RECORD_DTYPE)
    verts = np.empty(vcap, dtype=abi.VERT_COLOR_DTYPE)
    normals = np.empty((vcap, 3), dtype=np.float32) if params.outputs & abi.UWW_OUT_NORMALS else None
    inds = np.empty(icap, dtype=np.uint32)
    cases = np.zeros(nc, dtype=np.uint8) if params.outputs & abi.UWW_OUT_CASES else None
    samples = np.zeros(ns, dtype=np.float32) if params.outputs & abi.UWW_OUT_SAMPLES else None
    totals = np.zeros(4, dtype=np.uint64)

    def ptr(a):
        return a.ctypes.data if a is not None else None

    out = abi.MeshOut(ptr(verts), ptr(normals), ptr(inds), ptr(cases), ptr(samples), ptr(records), ptr(totals),
                      vcap, icap, cases.size if cases is not None else 0, samples.size if samples is not None else 0)
    sin = np.ascontiguousarray(samples_in, dtype=np.float32) if samples_in is not None else None
    st = lib().oracle_build_chunks(C.byref(params), precision, search, descs.ctypes.data_as(C.c_void_p), n,
                                   C.byref(out), threads, ptr(sin), sin.size if sin is not None else 0)
    if st not in (abi.UWW_OK, abi.UWW_ERR_CAPACITY):
        raise RuntimeError(f"oracle_build_chunks failed: {st}")
    nv, ni = min(int(totals[0]), vcap), min(int(totals[1]), icap)
    return MeshBatch(records, verts[:nv].copy(), normals[:nv].copy() if normals is not None else None,
                     inds[:ni].copy(), cases, totals, st, samples)


def sample_grid(params: abi.Params, desc, precision: int = F32) -> np.ndarray:
    d = np.ascontiguousarray(np.asarray(desc, dtype=abi.CHUNK_DESC_DTYPE).reshape(1))
    S = int(d["cells"][0]) + 1
    out = np.zeros(S ** 3, dtype=np.float32)
    st = lib().oracle_sample_grid(C.byref(params), precision, d.ctypes.data_as(C.c_void_p),
                                  out.ctypes.data_as(C.c_void_p))
    if st:
        raise RuntimeError(f"oracle_sample_grid failed: {st}")
    return out


def density_at(params: abi.Params, xyz: np.ndarray, precision: int = F32, grad: bool = False):
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
