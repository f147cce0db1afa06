"""Per-frame chunk build as one CUDA graph, and the autotuner, over the C ABI.

The reference's World::build_step (world.rs:113-145) builds a slice of the
queued chunks each frame on the CPU.  :class:`FrameBuilder` builds the whole
frame's list in one graph launch (descriptor upload, persistent build,
record/total download) through ``uww_frame_*``; :func:`autotune` wraps
``uww_autotune``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check, lib
from .chunk import Context, DeviceArray, HostArray


class FrameBuilder:
    def __init__(self, ctx: Context, max_chunks: int, max_cells: int, vert_capacity: int, ind_capacity: int,
                 want_normals: bool = True):
        self.ctx = ctx
        self.max_chunks, self.max_cells = int(max_chunks), int(max_cells)
        self.vcap, self.icap = int(vert_capacity), int(ind_capacity)
        self.h_desc = HostArray((self.max_chunks,), abi.CHUNK_DESC_DTYPE)
        self.h_desc.array[:] = np.zeros(1, abi.CHUNK_DESC_DTYPE)
        self.h_count = HostArray((1,), np.uint32)
        self.h_count.array[0] = 0
        self.h_rec = HostArray((self.max_chunks,), abi.CHUNK_RECORD_DTYPE)
        self.h_tot = HostArray((4,), np.uint64)
        self.d_verts = DeviceArray(self.vcap * 24)
        self.d_norm = DeviceArray(self.vcap * 12) if want_normals else None
        self.d_inds = DeviceArray(self.icap * 4)
        self.d_rec = DeviceArray(self.max_chunks * 32)
        self.d_tot = DeviceArray(32)
        out = abi.MeshOut(self.d_verts.ptr, self.d_norm.ptr if self.d_norm else None, self.d_inds.ptr, None, None,
                          self.d_rec.ptr, self.d_tot.ptr, self.vcap, self.icap, 0, 0)
        h = C.c_void_p()
        check(lib().uww_frame_create(ctx.h, self.max_chunks, self.max_cells, C.c_void_p(self.h_desc.ptr),
                                     C.c_void_p(self.h_count.ptr), C.byref(out), C.c_void_p(self.h_rec.ptr),
                                     C.c_void_p(self.h_tot.ptr), C.byref(h)), "uww_frame_create")
        self.handle = h.value

    def submit(self, descs: np.ndarray):
        """Stage this frame's descriptors and launch the graph (asynchronous).
        The graph reads the staging buffer while it runs, so the previous
        frame must have finished (``ctx.sync()``, as :meth:`build` does)."""
        n = descs.shape[0]
        if n > self.max_chunks:
            raise ValueError(f"{n} chunks exceed the frame's maximum of {self.max_chunks}")
        self.h_desc.array[:n] = descs
        self.h_count.array[0] = n
        check(lib().uww_frame_launch(C.c_void_p(self.handle)), "uww_frame_launch")

    def build(self, descs: np.ndarray):
        """One frame: records (host copy) and totals of the first len(descs) chunks."""
        self.submit(descs)
        self.ctx.sync()
        n = descs.shape[0]
        return self.h_rec.array[:n].copy(), self.h_tot.array.copy()

    def set_params(self, p: abi.Params):
        check(lib().uww_frame_set_params(C.c_void_p(self.handle), C.byref(p)), "uww_frame_set_params")
        self.ctx.params = p

    def mesh(self, nv: int, ni: int):
        """Download the first nv vertices / ni indices of the last frame."""
        verts = self.ctx.download(self.d_verts, (nv,), abi.VERT_COLOR_DTYPE)
        norms = self.ctx.download(self.d_norm, (nv, 3), np.float32) if self.d_norm else None
        inds = self.ctx.download(self.d_inds, (ni,), np.uint32)
        return verts, norms, inds

    def close(self):
        if getattr(self, "handle", None):
            lib().uww_frame_destroy(C.c_void_p(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(ctx: Context, d_desc, n: int, max_cells: int, out: abi.MeshOut,
             cache_path: str | None = None) -> tuple[abi.Tuning, float]:
    """Run uww_autotune on device descriptors (a DeviceArray or a device address);
    returns the chosen tuning and its build time in µs."""
    t = abi.Tuning()
    us = C.c_float()
    ptr = d_desc.ptr if isinstance(d_desc, DeviceArray) else int(d_desc)
    check(lib().uww_autotune(ctx.h, C.c_void_p(ptr), n, max_cells, C.byref(out),
                             cache_path.encode() if cache_path else None, C.byref(t), C.byref(us)), "uww_autotune")
    return t, us.value
