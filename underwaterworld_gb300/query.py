"""Queries against a built batch: Chunk::tris_around and the boids' wall rays.

The reference's boids (boid.rs:175-244) gather the triangles of the cells
around each boid with ``Chunk::tris_around`` (chunk.rs:315-342) and cast a few
rays against them with ``util::Tri::intersects`` (util.rs:23-58).
:class:`RayScene` keeps a batch's mesh on the device with its per-cell
triangle offsets (``uww_cell_tri_offsets``) and a chunk-position index
(``uww_chunk_index``), and answers many boids' rays in one launch
(``uww_ray_query``): the nearest hit per ray, or -1.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check, lib
from .chunk import Context, DeviceArray, total_cells, totals_status

WALL_RANGE = 3  # boid.rs:15


class RayScene:
    def __init__(self, ctx: Context, descs: np.ndarray, vert_capacity: int = 1 << 20, ind_capacity: int = 1 << 22):
        if not ctx.params.outputs & abi.UWW_OUT_CASES:
            raise ValueError("the scene needs the per-cell cases (UWW_OUT_CASES)")
        self.ctx = ctx
        self.descs = np.ascontiguousarray(descs, dtype=abi.CHUNK_DESC_DTYPE)
        n = self.n = int(self.descs.shape[0])
        nc = total_cells(self.descs)
        self.d_desc = ctx.upload(self.descs)
        self.d_rec, self.d_tot = DeviceArray(n * 32), DeviceArray(32)
        self.d_verts, self.d_inds = DeviceArray(vert_capacity * 24), DeviceArray(ind_capacity * 4)
        self.d_cases, self.d_first = DeviceArray(nc), DeviceArray(nc * 4)
        self.table_size = 1 << max(4, int(2 * n - 1).bit_length())
        self.d_table = DeviceArray(self.table_size * 4)
        out = abi.MeshOut(self.d_verts.ptr, None, self.d_inds.ptr, self.d_cases.ptr, None, self.d_rec.ptr,
                          self.d_tot.ptr, vert_capacity, ind_capacity, nc, 0)
        L = lib()
        check(L.uww_build_chunks(ctx.h, C.c_void_p(self.d_desc.ptr), n, int(self.descs["cells"].max()), C.byref(out)),
              "uww_build_chunks")
        check(L.uww_cell_tri_offsets(ctx.h, C.c_void_p(self.d_desc.ptr), n, C.c_void_p(self.d_cases.ptr), nc,
                                     C.c_void_p(self.d_first.ptr)), "uww_cell_tri_offsets")
        check(L.uww_chunk_index(ctx.h, C.c_void_p(self.d_desc.ptr), n, C.c_void_p(self.d_table.ptr), self.table_size),
              "uww_chunk_index")
        ctx.sync()
        st = totals_status(ctx.download(self.d_tot, (4,), np.uint64))
        if st:
            raise abi.UWWError(st, "scene build")
        self.scene = abi.RayScene(self.d_desc.ptr, self.d_rec.ptr, self.d_verts.ptr, self.d_inds.ptr, self.d_cases.ptr,
                                  self.d_first.ptr, self.d_table.ptr, n, self.table_size)

    def cell_first(self) -> np.ndarray:
        return self.ctx.download(self.d_first, (total_cells(self.descs),), np.uint32)

    def batch(self):
        """Host copies of the scene's mesh (records, verts, inds, cases)."""
        from .chunk import MeshBatch
        tot = self.ctx.download(self.d_tot, (4,), np.uint64)
        nv, ni = int(tot[0]), int(tot[1])
        return MeshBatch(self.ctx.download(self.d_rec, (self.n,), abi.CHUNK_RECORD_DTYPE),
                         self.ctx.download(self.d_verts, (nv,), abi.VERT_COLOR_DTYPE), None,
                         self.ctx.download(self.d_inds, (ni,), np.uint32),
                         self.ctx.download(self.d_cases, (total_cells(self.descs),), np.uint8), tot, abi.UWW_OK)

    def cast(self, origins: np.ndarray, dirs: np.ndarray, rng: int = WALL_RANGE) -> np.ndarray:
        """Nearest hit distance per (query, ray), -1 where nothing is hit within rng."""
        origins = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
        nq = origins.shape[0]
        dirs = np.ascontiguousarray(dirs, dtype=np.float32).reshape(nq, -1, 3)
        nr = dirs.shape[1]
        d_o, d_d = self.ctx.upload(origins), self.ctx.upload(dirs)
        d_t = DeviceArray(nq * nr * 4)
        check(lib().uww_ray_query(self.ctx.h, C.byref(self.scene), C.c_void_p(d_o.ptr), nq, C.c_void_p(d_d.ptr), nr,
                                  rng, C.c_void_p(d_t.ptr)), "uww_ray_query")
        self.ctx.sync()
        return self.ctx.download(d_t, (nq, nr), np.float32)
