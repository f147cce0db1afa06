"""ctypes mirror of include/uww.h and the loader of libuww_gb300.so.

The library is loaded from the package's in-tree ``_build`` directory.  There
is no fallback: if the shared object is missing, :func:`lib` raises, and every
compute entry point returns ``UWW_ERR_CUDA`` when no GPU is present.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
LIB_PATH = PKG / "_build" / "libuww_gb300.so"
HEADER = ROOT / "include" / "uww.h"

# ---- constants (uww.h) ------------------------------------------------------
UWW_OK, UWW_ERR_INVALID_ARG, UWW_ERR_CUDA, UWW_ERR_CAPACITY, UWW_ERR_OOM, UWW_ERR_TIMEOUT = range(6)
UWW_MAX_OCTAVES = 16
UWW_MAX_CELLS = 64
UWW_BIAS_NONE, UWW_BIAS_TERRACED, UWW_BIAS_LINEAR = 0, 1, 2
UWW_MATH_EXACT, UWW_MATH_FAST = 0, 1
UWW_DEDUP_ORIENTED, UWW_DEDUP_EDGE = 0, 1
UWW_OUT_COLOR, UWW_OUT_NORMALS, UWW_OUT_CASES, UWW_OUT_SAMPLES = 1, 2, 4, 8
UWW_CHUNK_EARLY_BLANK, UWW_CHUNK_HAS_MESH, UWW_CHUNK_OVERFLOW = 1, 2, 4
UWW_ERRFLAG_TIMEOUT, UWW_ERRFLAG_BAD, UWW_ERRFLAG_RANGE = 1, 2, 4
H2D, D2H, D2D = 0, 1, 2


class Params(C.Structure):
    _fields_ = [
        ("seed", C.c_uint32), ("octaves", C.c_uint32), ("chunk_size", C.c_int32),
        ("base_freq", C.c_float), ("lacunarity", C.c_float), ("persistence", C.c_float),
        ("amplitude", C.c_float), ("normalize", C.c_int32), ("bias_mode", C.c_int32),
        ("bias_a", C.c_float), ("bias_b", C.c_float), ("bias_c", C.c_float),
        ("iso_level", C.c_float), ("offset", C.c_float * 3), ("explicit_amps", C.c_int32),
        ("amps", C.c_float * UWW_MAX_OCTAVES), ("math_mode", C.c_int32), ("dedup_mode", C.c_int32),
        ("outputs", C.c_uint32), ("color_min_z", C.c_float), ("color_max_z", C.c_float),
    ]

    def copy(self) -> "Params":
        q = Params()
        C.pointer(q)[0] = self
        return q


class ChunkDesc(C.Structure):
    _fields_ = [("pos", C.c_int32 * 3), ("cells", C.c_uint32), ("cell_offset", C.c_uint32),
                ("sample_offset", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class ChunkRecord(C.Structure):
    _fields_ = [("num_verts", C.c_uint32), ("num_inds", C.c_uint32), ("vert_offset", C.c_uint32),
                ("ind_offset", C.c_uint32), ("flags", C.c_uint32), ("num_active_cells", C.c_uint32),
                ("reserved", C.c_uint32 * 2)]


class MeshOut(C.Structure):
    _fields_ = [("verts", C.c_void_p), ("normals", C.c_void_p), ("inds", C.c_void_p), ("cases", C.c_void_p),
                ("samples", C.c_void_p), ("records", C.c_void_p), ("totals", C.c_void_p),
                ("vert_capacity", C.c_uint32), ("ind_capacity", C.c_uint32),
                ("case_capacity", C.c_uint64), ("sample_capacity", C.c_uint64)]


class RayScene(C.Structure):
    _fields_ = [("chunks", C.c_void_p), ("records", C.c_void_p), ("verts", C.c_void_p), ("inds", C.c_void_p),
                ("cases", C.c_void_p), ("cell_first", C.c_void_p), ("table", C.c_void_p), ("n", C.c_uint32),
                ("table_size", C.c_uint32)]


class ScheduleParams(C.Structure):
    _fields_ = [("sub_pos", C.c_float * 3), ("sub_chunk", C.c_int32 * 3), ("view_proj", C.c_float * 16),
                ("gen_proj", C.c_float * 16), ("generation_dist", C.c_int32), ("view_dist", C.c_int32),
                ("min_z", C.c_int32), ("max_z", C.c_int32), ("cells", C.c_uint32)]


class CameraUniform(C.Structure):
    _fields_ = [("view_proj", C.c_float * 16), ("fog_color", C.c_float * 3), ("pad1", C.c_float),
                ("sub_pos", C.c_float * 3), ("pad2", C.c_float), ("sub_forward", C.c_float * 3), ("pad3", C.c_float)]


class Tuning(C.Structure):
    _fields_ = [("threads", C.c_int32), ("blocks_per_sm", C.c_int32), ("smem_cells", C.c_int32),
                ("reserved", C.c_int32)]


assert C.sizeof(ChunkDesc) == 32 and C.sizeof(ChunkRecord) == 32

# numpy views of the structs
try:
    import numpy as np

    CHUNK_DESC_DTYPE = np.dtype([("pos", "<i4", 3), ("cells", "<u4"), ("cell_offset", "<u4"),
                                 ("sample_offset", "<u4"), ("reserved", "<u4", 2)])
    CHUNK_RECORD_DTYPE = np.dtype([("num_verts", "<u4"), ("num_inds", "<u4"), ("vert_offset", "<u4"),
                                   ("ind_offset", "<u4"), ("flags", "<u4"), ("num_active_cells", "<u4"),
                                   ("reserved", "<u4", 2)])
    VERT_COLOR_DTYPE = np.dtype([("pos", "<f4", 3), ("color", "<f4", 3)])
except ImportError:  # pragma: no cover
    np = None

P = C.c_void_p
_SIGS = {
    "uww_abi_version": (C.c_int, []),
    "uww_status_string": (C.c_char_p, [C.c_int]),
    "uww_last_error": (C.c_char_p, []),
    "uww_params_reference": (None, [C.POINTER(Params)]),
    "uww_perm_table": (C.c_int, [C.c_uint32, P]),
    "uww_layout_cells": (C.c_int, [P, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "uww_build_chunks_from_samples": (C.c_int, [P, P, C.c_uint32, C.c_uint32, P, C.c_uint64, C.POINTER(MeshOut)]),
    "uww_ctx_create": (C.c_int, [C.POINTER(Params), P, C.POINTER(P)]),
    "uww_ctx_destroy": (C.c_int, [P]),
    "uww_ctx_set_params": (C.c_int, [P, C.POINTER(Params)]),
    "uww_ctx_get_params": (C.c_int, [P, C.POINTER(Params)]),
    "uww_ctx_stream": (P, [P]),
    "uww_ctx_sync": (C.c_int, [P]),
    "uww_build_chunks": (C.c_int, [P, P, C.c_uint32, C.c_uint32, C.POINTER(MeshOut)]),
    "uww_build_chunk_plain": (C.c_int, [P, P, C.c_uint32, C.POINTER(MeshOut)]),
    "uww_build_chunks_noalloc": (C.c_int, [C.POINTER(Params), P, P, C.c_uint32, C.c_uint32, C.POINTER(MeshOut)]),
    "uww_build_chunks_host": (C.c_int, [P, P, C.c_uint32, C.POINTER(MeshOut)]),
    "uww_ctx_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "uww_ctx_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "uww_device_alloc": (C.c_int, [C.c_size_t, C.POINTER(P)]),
    "uww_device_free": (C.c_int, [P]),
    "uww_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(P)]),
    "uww_host_free": (C.c_int, [P]),
    "uww_memcpy": (C.c_int, [P, P, P, C.c_size_t, C.c_int]),
    "uww_memset": (C.c_int, [P, P, C.c_int, C.c_size_t]),
    "uww_density_at": (C.c_int, [P, P, C.c_uint32, P]),
    "uww_probe_fma": (C.c_int, [P, C.c_uint32, C.c_uint32, P, C.POINTER(C.c_double)]),
    "uww_autotune": (C.c_int, [P, P, C.c_uint32, C.c_uint32, C.POINTER(MeshOut), C.c_char_p, C.POINTER(Tuning),
                               C.POINTER(C.c_float)]),
    "uww_frame_create": (C.c_int, [P, C.c_uint32, C.c_uint32, P, P, C.POINTER(MeshOut), P, P, C.POINTER(P)]),
    "uww_frame_launch": (C.c_int, [P]),
    "uww_frame_set_params": (C.c_int, [P, C.POINTER(Params)]),
    "uww_frame_destroy": (C.c_int, [P]),
    "uww_sample_chunks": (C.c_int, [P, P, C.c_uint32, C.c_uint32, P, C.c_uint64]),
    "uww_sample_status": (C.c_int, [P, C.POINTER(C.c_uint32)]),
    "uww_cell_tri_offsets": (C.c_int, [P, P, C.c_uint32, P, C.c_uint64, P]),
    "uww_chunk_index": (C.c_int, [P, P, C.c_uint32, P, C.c_uint32]),
    "uww_ray_query": (C.c_int, [P, C.POINTER(RayScene), P, C.c_uint32, P, C.c_uint32, C.c_int32, P]),
    "uww_schedule_chunks": (C.c_int, [P, C.POINTER(ScheduleParams), P, P, P, C.c_uint32, P, C.c_uint32, P,
                                      C.c_uint32, P]),
    "uww_shade_vertices": (C.c_int, [P, C.POINTER(CameraUniform), P, P, C.c_uint32, C.c_uint32, P, P, P]),
    "uww_forward": (C.c_int, [P, P, C.c_uint32, C.c_uint32, C.POINTER(MeshOut), P]),
    "uww_backward": (C.c_int, [P, P, C.c_uint32, C.c_uint32, P, P, P, P, P, C.c_uint64]),
    "uww_height_loss": (C.c_int, [P, P, P, C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_uint32, C.c_uint32,
                                  P, P, P, P]),
}


def theta_count(octaves: int) -> int:
    """UWW_THETA_COUNT: per-octave amplitudes, base frequency, offset xyz, iso level."""
    return int(octaves) + 5

_lib = None


class UWWError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status) if _lib is not None else str(status)
        if _lib is not None and status in (UWW_ERR_CUDA, UWW_ERR_OOM):
            msg += " [" + _lib.uww_last_error().decode() + "]"
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


def declared_functions() -> list[str]:
    """Function names declared in include/uww.h."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(uww_[a-z0-9_]+)\s*\(", text)))


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m underwaterworld_gb300.build` "
                "(there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def status_string(s: int) -> str:
    return lib().uww_status_string(s).decode()


def check(status: int, what: str = "") -> None:
    if status != UWW_OK:
        raise UWWError(status, what)


def reference_params() -> Params:
    p = Params()
    lib().uww_params_reference(C.byref(p))
    return p


def perm_table(seed: int):
    buf = (C.c_uint8 * 256)()
    check(lib().uww_perm_table(seed, buf), "uww_perm_table")
    return bytes(buf)
