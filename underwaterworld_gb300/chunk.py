"""Host-side mirror of the reference's chunk-build interface over the C ABI.

Reference interface (LelsersLasers/UnderwaterWorld, underwater_world/src/):
  * ``noise::Perlin::new(seed)`` (state.rs:359)          -> :class:`Context`
  * ``perlin_util::iso_at(perlin, x, y, z)`` (perlin_util.rs:24-29) -> :meth:`Context.iso_at`
  * ``Chunk::new(pos)`` / ``build_full`` / ``build_partial`` (chunk.rs:89-103,266-313)
                                                          -> :class:`Chunk`
  * ``Chunk::not_blank`` / ``num_inds`` / buffer slices (chunk.rs:344-348)
  * ``World``'s one-chunk-per-frame loop (world.rs:113-145) -> :meth:`Context.build_chunks`

Everything runs in libuww_gb300.so; there is no CPU path here.
"""
from __future__ import annotations

import ctypes as C
import numpy as np

from . import abi
from .abi import check, lib
from .layout import (CHUNK_SIZE, INTERNAL_SIZE, MeshBatch, make_descs, total_cells,  # noqa: F401
                     total_samples, totals_status)


class DeviceArray:
    """A raw device allocation made through uww_device_alloc."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = C.c_void_p()
        check(lib().uww_device_alloc(max(self.nbytes, 1), C.byref(p)), "uww_device_alloc")
        self.ptr = p.value

    def free(self):
        if self.ptr:
            lib().uww_device_free(C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class HostArray:
    """Page-locked host memory (uww_host_alloc) viewed as a numpy array."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        p = C.c_void_p()
        check(lib().uww_host_alloc(max(n, 1), C.byref(p)), "uww_host_alloc")
        self.ptr = p.value
        self.nbytes = n
        buf = (C.c_uint8 * max(n, 1)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=np.uint8, count=n).view(dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            lib().uww_host_free(C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """A noise::Perlin handle plus the chunk builder, on one CUDA stream."""

    def __init__(self, params: abi.Params | None = None, stream: int | None = None):
        self.params = params if params is not None else abi.reference_params()
        h = C.c_void_p()
        check(lib().uww_ctx_create(C.byref(self.params), C.c_void_p(stream), C.byref(h)), "uww_ctx_create")
        self.handle = h.value

    def close(self):
        if getattr(self, "handle", None):
            lib().uww_ctx_destroy(C.c_void_p(self.handle))
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def h(self):
        return C.c_void_p(self.handle)

    def set_params(self, params: abi.Params):
        check(lib().uww_ctx_set_params(self.h, C.byref(params)), "uww_ctx_set_params")
        self.params = params

    def set_tuning(self, threads=0, blocks_per_sm=0, smem_cells=0, options=None):
        """Launch shape (0 = automatic) and, when given, the UWW_TUNE_* options;
        the spin limit and test flags stay as they are."""
        t = abi.Tuning()
        check(lib().uww_ctx_get_tuning(self.h, C.byref(t)), "uww_ctx_get_tuning")
        t.threads, t.blocks_per_sm, t.smem_cells = threads, blocks_per_sm, smem_cells
        if options is not None:
            t.options = options
        check(lib().uww_ctx_set_tuning(self.h, C.byref(t)), "uww_ctx_set_tuning")

    def launch_shape(self, n: int, max_cells: int) -> abi.LaunchShape:
        """The launch shape of a batched build of n chunks of up to max_cells
        cells per edge (uww_launch_shape_of): which build, slabs per chunk,
        threads, grid, CTAs per SM, dynamic shared memory."""
        s = abi.LaunchShape()
        check(lib().uww_launch_shape_of(self.h, n, max_cells, C.byref(s)), "uww_launch_shape_of")
        return s

    def stream(self) -> int:
        return lib().uww_ctx_stream(self.h) or 0

    def sync(self):
        check(lib().uww_ctx_sync(self.h), "uww_ctx_sync")

    # -- memory helpers ---------------------------------------------------------
    def upload(self, arr: np.ndarray) -> DeviceArray:
        arr = np.ascontiguousarray(arr)
        d = DeviceArray(arr.nbytes)
        check(lib().uww_memcpy(self.h, C.c_void_p(d.ptr), arr.ctypes.data_as(C.c_void_p), arr.nbytes, abi.H2D), "upload")
        self.sync()
        return d

    def download(self, d: DeviceArray, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        if out.nbytes:
            check(lib().uww_memcpy(self.h, out.ctypes.data_as(C.c_void_p), C.c_void_p(d.ptr), out.nbytes, abi.D2H), "download")
            self.sync()
        return out

    # -- builds -----------------------------------------------------------------
    def build_chunks(self, descs: np.ndarray, vert_capacity: int, ind_capacity: int, want_normals=None,
                     want_cases=None) -> MeshBatch:
        """Host-buffer batched build (uww_build_chunks_host)."""
        descs = np.ascontiguousarray(descs, dtype=abi.CHUNK_DESC_DTYPE)
        n = descs.shape[0]
        outputs = self.params.outputs
        want_normals = bool(outputs & abi.UWW_OUT_NORMALS) if want_normals is None else want_normals
        want_cases = bool(outputs & abi.UWW_OUT_CASES) if want_cases is None else want_cases
        want_samples = bool(outputs & abi.UWW_OUT_SAMPLES)
        records = np.zeros(n, dtype=abi.CHUNK_RECORD_DTYPE)
        verts = np.zeros(vert_capacity, dtype=abi.VERT_COLOR_DTYPE)
        normals = np.zeros((vert_capacity, 3), dtype=np.float32) if want_normals else None
        inds = np.zeros(ind_capacity, dtype=np.uint32)
        cases = np.zeros(total_cells(descs), dtype=np.uint8) if want_cases else None
        samples = np.zeros(total_samples(descs), dtype=np.float32) if want_samples else None
        totals = np.zeros(4, dtype=np.uint64)

        def ptr(a):
            return a.ctypes.data if a is not None else None

        out = abi.MeshOut(ptr(verts), ptr(normals), ptr(inds), ptr(cases), ptr(samples), ptr(records),
                          ptr(totals), vert_capacity, ind_capacity, cases.size if cases is not None else 0,
                          samples.size if samples is not None else 0)
        st = lib().uww_build_chunks_host(self.h, descs.ctypes.data_as(C.c_void_p), n, C.byref(out))
        if st not in (abi.UWW_OK, abi.UWW_ERR_CAPACITY):
            raise abi.UWWError(st, "uww_build_chunks_host")
        nv, ni = min(int(totals[0]), vert_capacity), min(int(totals[1]), ind_capacity)
        return MeshBatch(records, verts[:nv], normals[:nv] if normals is not None else None, inds[:ni], cases,
                         totals, st, samples)

    def build_chunks_device(self, descs: np.ndarray, vert_capacity: int, ind_capacity: int,
                            samples_in: np.ndarray | None = None) -> MeshBatch:
        """Device-buffer batched build (uww_build_chunks, or uww_build_chunks_from_samples
        when samples_in is given): uploads, launches, downloads."""
        descs = np.ascontiguousarray(descs, dtype=abi.CHUNK_DESC_DTYPE)
        n = descs.shape[0]
        outputs = self.params.outputs
        want_normals = bool(outputs & abi.UWW_OUT_NORMALS)
        want_cases = bool(outputs & abi.UWW_OUT_CASES)
        want_samples = bool(outputs & abi.UWW_OUT_SAMPLES)
        ncells, nsamp = total_cells(descs), total_samples(descs)
        d_desc = self.upload(descs) if n else DeviceArray(32)
        d_rec = DeviceArray(max(n, 1) * 32)
        d_verts = DeviceArray(vert_capacity * 24)
        d_norm = DeviceArray(vert_capacity * 12) if want_normals else None
        d_inds = DeviceArray(ind_capacity * 4)
        d_cases = DeviceArray(ncells) if want_cases else None
        d_samp = DeviceArray(nsamp * 4) if want_samples else None
        d_tot = DeviceArray(32)
        out = abi.MeshOut(d_verts.ptr, d_norm.ptr if d_norm else None, d_inds.ptr, d_cases.ptr if d_cases else None,
                          d_samp.ptr if d_samp else None, d_rec.ptr, d_tot.ptr, vert_capacity, ind_capacity,
                          ncells if d_cases else 0, nsamp if d_samp else 0)
        max_cells = int(descs["cells"].max()) if n else 1
        if samples_in is not None:
            sin = np.ascontiguousarray(samples_in, dtype=np.float32)
            d_in = self.upload(sin)
            check(lib().uww_build_chunks_from_samples(self.h, C.c_void_p(d_desc.ptr), n, max_cells,
                                                      C.c_void_p(d_in.ptr), sin.size, C.byref(out)),
                  "uww_build_chunks_from_samples")
        else:
            check(lib().uww_build_chunks(self.h, C.c_void_p(d_desc.ptr), n, max_cells, C.byref(out)),
                  "uww_build_chunks")
        self.sync()
        totals = self.download(d_tot, (4,), np.uint64)
        nv, ni = min(int(totals[0]), vert_capacity), min(int(totals[1]), ind_capacity)
        records = self.download(d_rec, (n,), abi.CHUNK_RECORD_DTYPE)
        verts = self.download(d_verts, (nv,), abi.VERT_COLOR_DTYPE)
        normals = self.download(d_norm, (nv, 3), np.float32) if d_norm else None
        inds = self.download(d_inds, (ni,), np.uint32)
        cases = self.download(d_cases, (ncells,), np.uint8) if d_cases else None
        samples = self.download(d_samp, (nsamp,), np.float32) if d_samp else None
        return MeshBatch(records, verts, normals, inds, cases, totals, totals_status(totals), samples)

    def sample_chunks(self, descs: np.ndarray) -> np.ndarray:
        """Density samples of every chunk (uww_sample_chunks, Chunk::build_iso for a
        batch), laid out at each descriptor's sample_offset."""
        descs = np.ascontiguousarray(descs, dtype=abi.CHUNK_DESC_DTYPE)
        n = descs.shape[0]
        ns = total_samples(descs)
        d_desc = self.upload(descs) if n else DeviceArray(32)
        d_s = DeviceArray(max(ns, 1) * 4)
        max_cells = int(descs["cells"].max()) if n else 1
        check(lib().uww_sample_chunks(self.h, C.c_void_p(d_desc.ptr), n, max_cells, C.c_void_p(d_s.ptr), ns),
              "uww_sample_chunks")
        flags = C.c_uint32()
        check(lib().uww_sample_status(self.h, C.byref(flags)), "uww_sample_status")
        if flags.value:
            raise abi.UWWError(abi.UWW_ERR_INVALID_ARG, f"uww_sample_chunks flags {flags.value}")
        return self.download(d_s, (ns,), np.float32)

    def density_at(self, xyz: np.ndarray) -> np.ndarray:
        """Density at world points (n, 3) f32 -- iso_at with world = chunk units * CHUNK_SIZE."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        n = xyz.shape[0]
        if n == 0:
            return np.zeros(0, dtype=np.float32)
        d_in = self.upload(xyz)
        d_out = DeviceArray(n * 4)
        check(lib().uww_density_at(self.h, C.c_void_p(d_in.ptr), n, C.c_void_p(d_out.ptr)), "uww_density_at")
        self.sync()
        return self.download(d_out, (n,), np.float32)

    def iso_at(self, x: float, y: float, z: float) -> float:
        """perlin_util::iso_at(perlin, x, y, z) with (x, y, z) in chunk units (perlin_util.rs:24)."""
        cs = self.params.chunk_size
        return float(self.density_at(np.array([[x * cs, y * cs, z * cs]], dtype=np.float32))[0])


class Chunk:
    """Mirror of ``chunk::Chunk`` (chunk.rs:80-349) built by one plain launch.

    ``Chunk(pos)`` records the chunk position (chunk.rs:89-103); ``build_full``
    runs the whole build (chunk.rs:266-268) as one kernel launch on the
    context's stream; the accessors follow chunk.rs:344-348.
    """

    def __init__(self, pos, cells: int = INTERNAL_SIZE):
        self.pos = tuple(int(v) for v in pos)
        self.cells = int(cells)
        self.chunk_offset = tuple(v * CHUNK_SIZE for v in self.pos)
        self._verts = None
        self._normals = None
        self._inds = None
        self._record = None
        self._done = False

    @classmethod
    def new(cls, pos):
        return cls(pos)

    def build_full(self, ctx: Context):
        d = make_descs([self.pos], self.cells)
        # at most 5 triangles per cell, and never more vertices than indices
        vcap = icap = 15 * self.cells ** 3
        d_desc = ctx.upload(d)
        d_rec, d_tot = DeviceArray(32), DeviceArray(32)
        d_verts, d_inds = DeviceArray(vcap * 24), DeviceArray(icap * 4)
        want_normals = bool(ctx.params.outputs & abi.UWW_OUT_NORMALS)
        d_norm = DeviceArray(vcap * 12) if want_normals else None
        out = abi.MeshOut(d_verts.ptr, d_norm.ptr if d_norm else None, d_inds.ptr, None, None, d_rec.ptr,
                          d_tot.ptr, vcap, icap)
        check(lib().uww_build_chunk_plain(ctx.h, C.c_void_p(d_desc.ptr), self.cells, C.byref(out)),
              "uww_build_chunk_plain")
        ctx.sync()
        st = totals_status(ctx.download(d_tot, (4,), np.uint64))
        if st:
            raise abi.UWWError(st, "uww_build_chunk_plain")
        self._record = ctx.download(d_rec, (1,), abi.CHUNK_RECORD_DTYPE)[0]
        nv, ni = int(self._record["num_verts"]), int(self._record["num_inds"])
        self._verts = ctx.download(d_verts, (nv,), abi.VERT_COLOR_DTYPE)
        self._normals = ctx.download(d_norm, (nv, 3), np.float32) if d_norm else None
        self._inds = ctx.download(d_inds, (ni,), np.uint32)
        self._done = True

    def build_partial(self, ctx: Context) -> bool:
        """The whole build is one launch, so the first call finishes it (chunk.rs:270)."""
        if not self._done:
            self.build_full(ctx)
        return True

    def not_blank(self) -> bool:
        return self._done and int(self._record["num_inds"]) > 0

    def num_inds(self) -> int:
        return int(self._record["num_inds"]) if self._done else 0

    def verts(self) -> np.ndarray:
        return self._verts

    def normals(self):
        return self._normals

    def inds(self) -> np.ndarray:
        return self._inds

    def inds_u16(self) -> np.ndarray:
        """The reference's u16 index buffer (state.rs:506); valid while ids < 65536."""
        if self._inds.size and int(self._inds.max()) > 0xFFFF:
            raise OverflowError("chunk has more than 65536 vertices; use the u32 indices")
        return self._inds.astype(np.uint16)

    def early_blank(self) -> bool:
        return self._done and bool(int(self._record["flags"]) & abi.UWW_CHUNK_EARLY_BLANK)
