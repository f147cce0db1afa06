"""Constants, struct layouts and parameter presets of include/uww.h, in pure Python.

Nothing here loads libuww_gb300.so: the CPU oracle and the benchmark's
reference arm describe their inputs and outputs with these layouts without
mapping the GPU library into their process.  :mod:`.abi` re-exports all of it
and adds the library binding.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

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

CHUNK_SIZE = 16       # chunk.rs:5
INTERNAL_SIZE = 12    # chunk.rs:6


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
                ("spin_limit", C.c_int32), ("test_flags", C.c_uint32), ("options", C.c_uint32),
                ("reserved", C.c_int32 * 2)]


UWW_TEST_WITHHOLD_FIRST = 1
UWW_TEST_WITHHOLD_RECORDS = 2
UWW_TUNE_NO_DEPTH_SHORTCUT = 1
UWW_TUNE_PIPELINED = 2


class LaunchShape(C.Structure):
    _fields_ = [("build", C.c_uint32), ("slabs_per_chunk", C.c_uint32), ("threads", C.c_uint32),
                ("grid", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("dyn_smem", C.c_uint32)]


UWW_BUILD_PIPELINED = 0
UWW_BUILD_SPLIT = 1


assert C.sizeof(ChunkDesc) == 32 and C.sizeof(ChunkRecord) == 32 and C.sizeof(Tuning) == 32

CHUNK_DESC_DTYPE = np.dtype([("pos", "<i4", 3), ("cells", "<u4"), ("cell_offset", "<u4"),
                             ("sample_offset", "<u4"), ("reserved", "<u4", 2)])
CHUNK_RECORD_DTYPE = np.dtype([("num_verts", "<u4"), ("num_inds", "<u4"), ("vert_offset", "<u4"),
                               ("ind_offset", "<u4"), ("flags", "<u4"), ("num_active_cells", "<u4"),
                               ("reserved", "<u4", 2)])
VERT_COLOR_DTYPE = np.dtype([("pos", "<f4", 3), ("color", "<f4", 3)])


def theta_count(octaves: int) -> int:
    """UWW_THETA_COUNT: per-octave amplitudes, base frequency, offset xyz, iso level."""
    return int(octaves) + 5


def reference_params() -> Params:
    """The reference's world constants, as uww_params_reference() fills them:
    PERLIN_OCTAVES = 3 (chunk.rs:9), CHUNK_SIZE = 16 (chunk.rs:5), noise input
    (local + offset) / CHUNK_SIZE (chunk.rs:108), lacunarity 2, persistence
    0.5, amplitude 1 and the amplitude-sum normalisation (perlin_util.rs:9-21),
    the terraced iso_at bias with MAX_HEIGHT = 32 and ADJ_Z_MOD = 0.25
    (perlin_util.rs:24-29, chunk.rs:11-12), ISO_LEVEL = -0.1 (chunk.rs:10),
    colour ramp between world::MIN_Z = -2 and MAX_Z = 2 (world.rs:11-12);
    seed 0, the parity build, oriented dedup, colour output."""
    p = Params()
    p.seed = 0
    p.octaves = 3
    p.chunk_size = CHUNK_SIZE
    p.base_freq = 1.0 / 16.0
    p.lacunarity = 2.0
    p.persistence = 0.5
    p.amplitude = 1.0
    p.normalize = 1
    p.bias_mode = UWW_BIAS_TERRACED
    p.bias_a = 16.0
    p.bias_b = 32.0
    p.bias_c = 0.25
    p.iso_level = -0.1
    p.math_mode = UWW_MATH_EXACT
    p.dedup_mode = UWW_DEDUP_ORIENTED
    p.outputs = UWW_OUT_COLOR
    p.color_min_z = -2.0
    p.color_max_z = 2.0
    return p


def make_descs(positions, cells) -> np.ndarray:
    """Chunk descriptors with cell and sample offsets laid out in order (uww_layout_cells)."""
    positions = np.asarray(positions, dtype=np.int32).reshape(-1, 3)
    cells = np.broadcast_to(np.asarray(cells, dtype=np.uint32), (positions.shape[0],))
    d = np.zeros(positions.shape[0], dtype=CHUNK_DESC_DTYPE)
    d["pos"] = positions
    d["cells"] = cells
    c3 = cells.astype(np.uint64) ** 3
    s3 = (cells.astype(np.uint64) + 1) ** 3
    d["cell_offset"] = (np.cumsum(c3) - c3).astype(np.uint32)
    d["sample_offset"] = (np.cumsum(s3) - s3).astype(np.uint32)
    return d


def total_cells(descs) -> int:
    return int((descs["cells"].astype(np.uint64) ** 3).sum()) if len(descs) else 0


def total_samples(descs) -> int:
    return int(((descs["cells"].astype(np.uint64) + 1) ** 3).sum()) if len(descs) else 0


def totals_status(totals) -> int:
    """Status of a finished device build from its totals words."""
    flags = int(totals[3])
    if flags & UWW_ERRFLAG_TIMEOUT:
        return UWW_ERR_TIMEOUT
    if flags & (UWW_ERRFLAG_BAD | UWW_ERRFLAG_RANGE):
        return UWW_ERR_INVALID_ARG
    if int(totals[2]):
        return UWW_ERR_CAPACITY
    return UWW_OK


@dataclass
class MeshBatch:
    """Outputs of a batched build, in chunk order."""
    records: np.ndarray          # CHUNK_RECORD_DTYPE
    verts: np.ndarray            # VERT_COLOR_DTYPE
    normals: np.ndarray | None   # (V, 3) f32
    inds: np.ndarray             # u32, chunk-local vertex ids
    cases: np.ndarray | None     # u8 per cell
    totals: np.ndarray           # u64[4]
    status: int
    samples: np.ndarray | None = None  # f32 density samples per chunk

    def chunk(self, i: int):
        r = self.records[i]
        v0, nv, i0, ni = int(r["vert_offset"]), int(r["num_verts"]), int(r["ind_offset"]), int(r["num_inds"])
        nrm = self.normals[v0:v0 + nv] if self.normals is not None else None
        return self.verts[v0:v0 + nv], nrm, self.inds[i0:i0 + ni]
