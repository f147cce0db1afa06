"""The chunk scheduler's feed (World::update_nearby, world.rs:148-234) on the GPU.

:func:`frustum_matrix` is camera.rs:58-62 (OPENGL_TO_WGPU * perspective *
look_at_rh, column-major like cgmath), computed on the host as the reference
does.  :class:`Scheduler` runs ``uww_schedule_chunks``: the generation list
comes back as device descriptors in GenPrio order, ready to be the batched
build's input (its work queue takes them in order, so in-view chunks finish
first), and the render list as chunk positions.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import abi
from .abi import check, lib
from .chunk import Context, DeviceArray

VIEW_DIST, GENERATION_DIST = 4, 5        # world.rs:8-9
MIN_Z, MAX_Z = -2, 2                     # world.rs:11-12
VIEW_FRUST_FOVY, GENERATE_FRUST_FOVY = 55.0, 90.0   # world.rs:16-17
Z_NEAR = 2.0                             # camera.rs:4
Z_FAR = 16.0 * (VIEW_DIST + 1)           # camera.rs:5

OPENGL_TO_WGPU = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0.5, 0], [0, 0, 0.5, 1]], np.float32)  # columns


def _cols(m):
    return np.asarray(m, np.float32)


def perspective(fovy_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """cgmath::perspective, columns as rows of the returned array."""
    f = np.float32(1.0 / math.tan(math.radians(fovy_deg) / 2.0))
    m = np.zeros((4, 4), np.float32)
    m[0, 0] = f / np.float32(aspect)
    m[1, 1] = f
    m[2, 2] = np.float32((far + near) / (near - far))
    m[2, 3] = -1.0
    m[3, 2] = np.float32(2.0 * far * near / (near - far))
    return m


def look_at_rh(eye, target, up) -> np.ndarray:
    eye, target, up = (np.asarray(v, np.float32) for v in (eye, target, up))
    f = target - eye
    f = f / np.float32(np.linalg.norm(f))
    s = np.cross(f, up)
    s = s / np.float32(np.linalg.norm(s))
    u = np.cross(s, f)
    m = np.zeros((4, 4), np.float32)
    m[0, :3] = [s[0], u[0], -f[0]]
    m[1, :3] = [s[1], u[1], -f[1]]
    m[2, :3] = [s[2], u[2], -f[2]]
    m[3, :3] = [-np.dot(eye, s), -np.dot(eye, u), np.dot(eye, f)]
    m[3, 3] = 1.0
    return m


def matmul_cols(a, b) -> np.ndarray:
    """Product of two column-major matrices stored as arrays of columns."""
    return (np.asarray(b, np.float32) @ np.asarray(a, np.float32)).astype(np.float32)


def frustum_matrix(eye, target, up, fovy: float, aspect: float) -> np.ndarray:
    """Camera::chunk_generation_frustum_matrix (camera.rs:58-62), 16 floats column-major."""
    view = look_at_rh(eye, target, up)
    proj = perspective(fovy, aspect, Z_NEAR, Z_FAR)
    return matmul_cols(OPENGL_TO_WGPU, matmul_cols(proj, view)).reshape(16)


def schedule_params(sub_pos, eye, target, up=(0.0, 0.0, 1.0), aspect: float = 16 / 9, cells: int = 12,
                    chunk_size: int = 16) -> abi.ScheduleParams:
    sp = abi.ScheduleParams()
    for i in range(3):
        sp.sub_pos[i] = float(np.float32(sub_pos[i]))
        sp.sub_chunk[i] = int(math.floor(np.float32(sub_pos[i]) / np.float32(chunk_size)))  # sub.rs:457-463
    for i, v in enumerate(frustum_matrix(eye, target, up, VIEW_FRUST_FOVY, aspect)):
        sp.view_proj[i] = float(v)
    for i, v in enumerate(frustum_matrix(eye, target, up, GENERATE_FRUST_FOVY, aspect)):
        sp.gen_proj[i] = float(v)
    sp.generation_dist, sp.view_dist, sp.min_z, sp.max_z, sp.cells = GENERATION_DIST, VIEW_DIST, MIN_Z, MAX_Z, cells
    return sp


class Scheduler:
    """Device buffers of the two lists; `known` is a built scene's device state."""

    def __init__(self, ctx: Context, capacity: int = 4096):
        self.ctx = ctx
        self.capacity = capacity
        self.d_gen = DeviceArray(capacity * 32)
        self.d_render = DeviceArray(capacity * 12)
        self.d_counts = DeviceArray(8)

    def run(self, sp: abi.ScheduleParams, known=None):
        """known: (d_descs, d_records, d_table, table_size) of the chunks already built, or None."""
        kd = kr = kt = None
        ts = 0
        if known is not None:
            kd, kr, kt, ts = (C.c_void_p(known[0]), C.c_void_p(known[1]), C.c_void_p(known[2]), known[3])
        check(lib().uww_schedule_chunks(self.ctx.h, C.byref(sp), kd, kr, kt, ts, C.c_void_p(self.d_gen.ptr),
                                        self.capacity, C.c_void_p(self.d_render.ptr), self.capacity,
                                        C.c_void_p(self.d_counts.ptr)), "uww_schedule_chunks")

    def fetch(self):
        counts = self.ctx.download(self.d_counts, (2,), np.uint32)
        ng, nr = min(int(counts[0]), self.capacity), min(int(counts[1]), self.capacity)
        gen = self.ctx.download(self.d_gen, (ng,), abi.CHUNK_DESC_DTYPE)
        ren = self.ctx.download(self.d_render, (nr, 3), np.int32)
        return gen, ren, counts
