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

# Constants, struct layouts and numpy dtypes live in .layout (no library load).
from .layout import *  # noqa: F401,F403
from .layout import (CHUNK_DESC_DTYPE, CHUNK_RECORD_DTYPE, VERT_COLOR_DTYPE, UWW_ERR_CUDA,  # noqa: F401
                     UWW_ERR_OOM, UWW_MAX_OCTAVES, UWW_OK, CameraUniform, ChunkDesc, ChunkRecord, MeshOut,
                     Params, RayScene, ScheduleParams, Tuning, LaunchShape, theta_count)

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
    "uww_launch_shape_of": (C.c_int, [P, C.c_uint32, C.c_uint32, C.POINTER(LaunchShape)]),
    "uww_device_alloc": (C.c_int, [C.c_size_t, C.POINTER(P)]),
    "uww_device_free": (C.c_int, [P]),
    "uww_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(P)]),
    "uww_host_free": (C.c_int, [P]),
    "uww_memcpy": (C.c_int, [P, P, P, C.c_size_t, C.c_int]),
    "uww_memset": (C.c_int, [P, P, C.c_int, C.c_size_t]),
    "uww_density_at": (C.c_int, [P, P, C.c_uint32, P]),
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
    """uww_params_reference() of the library (the same values as layout.reference_params)."""
    p = Params()
    lib().uww_params_reference(C.byref(p))
    return p


def perm_table(seed: int):
    buf = (C.c_uint8 * 256)()
    check(lib().uww_perm_table(seed, buf), "uww_perm_table")
    return bytes(buf)
