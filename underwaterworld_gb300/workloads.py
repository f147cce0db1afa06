"""Seeded synthetic chunk workloads (the benchmark and parity configurations).

* ``reference_grid``  -- 5x5x5 = 125 chunks centred on the origin, 12^3 cells,
  the reference's own world function and constants (chunk.rs:5-17,
  perlin_util.rs:6-29), permutation seed 0; iso-level -0.1 (the reference's
  ISO_LEVEL) or 0.
* ``uniform_grid``    -- 16x16x16 = 4096 chunks (positions 0..15 per axis) of
  12^3 cells; 4-octave fBm (base frequency 0.04 per world unit, lacunarity 2,
  persistence 0.5, amplitude 1) minus 0.03 * (z - 128); iso-level 0.
* ``mixed_lod``       -- 2048 chunks whose resolution is drawn per chunk from
  {12: 50%, 24: 35%, 48: 15%}, positions drawn without replacement from a
  64x64x16-chunk region (z from -8 to 7, so the surface near z = 0 lies
  inside it); 6-octave fBm (frequency 0.03) plus 0.02 * z; iso-level 0.
* ``adjoint_batch``   -- 8x8x8 = 512 chunks of 24^3 cells across the surface
  of the uniform grid's density (x, y 0..7, z 4..11), 4-octave fBm, for the
  adjoint check; ``cotangents`` gives its per-vertex dL/dp ~ N(0, I3) seeded
  by (chunk id, edge id).
"""
from __future__ import annotations

import numpy as np

from . import layout
from .layout import make_descs


def reference_grid(iso_level: float = -0.1, seed: int = 0, outputs: int = layout.UWW_OUT_COLOR):
    p = layout.reference_params()
    p.seed = seed
    p.iso_level = iso_level
    p.outputs = outputs
    g = np.arange(-2, 3)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    return p, make_descs(pos, 12)


def fbm_params(seed: int, octaves: int, freq: float, slope: float, z0: float, iso: float = 0.0,
               outputs: int = layout.UWW_OUT_COLOR) -> layout.Params:
    p = layout.reference_params()
    p.seed = seed
    p.octaves = octaves
    p.base_freq = freq
    p.lacunarity = 2.0
    p.persistence = 0.5
    p.amplitude = 1.0
    p.normalize = 1
    p.bias_mode = layout.UWW_BIAS_LINEAR
    p.bias_a = slope
    p.bias_b = z0
    p.bias_c = 0.0
    p.iso_level = iso
    p.outputs = outputs
    return p


def uniform_grid(seed: int = 0, side: int = 16, outputs: int = layout.UWW_OUT_COLOR):
    p = fbm_params(seed, 4, 0.04, -0.03, 128.0, 0.0, outputs)
    g = np.arange(side)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    return p, make_descs(pos, 12)


def mixed_lod(seed: int = 0, n: int = 2048, outputs: int = layout.UWW_OUT_COLOR):
    p = fbm_params(seed, 6, 0.03, 0.02, 0.0, 0.0, outputs)
    rng = np.random.default_rng(1000 + seed)
    flat = rng.choice(64 * 64 * 16, size=n, replace=False)
    pos = np.stack([flat // (64 * 16) - 32, (flat // 16) % 64 - 32, flat % 16 - 8], -1)
    cells = rng.choice(np.array([12, 24, 48]), size=n, p=[0.5, 0.35, 0.15])
    return p, make_descs(pos, cells)


def adjoint_batch(seed: int = 0, side: int = 8, cells: int = 24, outputs: int = layout.UWW_OUT_CASES):
    p = fbm_params(seed, 4, 0.04, -0.03, 128.0, 0.0, outputs)
    g = np.arange(side)
    pos = np.stack(np.meshgrid(g, g, g + 8 - side // 2, indexing="ij"), -1).reshape(-1, 3)
    return p, make_descs(pos, cells)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))


def cotangents(records: np.ndarray, edge_ids: np.ndarray, seed: int = 0) -> np.ndarray:
    """Per-vertex cotangents c_v ~ N(0, I3), a function of (seed, chunk id, edge
    id) only: splitmix64 counters, Box-Muller.  Shape (num_verts, 3), f32."""
    nv = edge_ids.size
    chunk = np.zeros(nv, dtype=np.uint64)
    for i, r in enumerate(records):
        o, n = int(r["vert_offset"]), int(r["num_verts"])
        if n and not (int(r["flags"]) & layout.UWW_CHUNK_OVERFLOW):
            chunk[o:o + n] = i
    with np.errstate(over="ignore"):
        key = (np.uint64(seed) << np.uint64(56)) ^ (chunk << np.uint64(32)) ^ edge_ids.astype(np.uint64)
        u = []
        for j in range(4):
            h = _splitmix64(key * np.uint64(4) + np.uint64(j))
            u.append(((h >> np.uint64(11)).astype(np.float64) + 0.5) / float(1 << 53))
    r0, r1 = np.sqrt(-2 * np.log(u[0])), np.sqrt(-2 * np.log(u[2]))
    c = np.stack([r0 * np.cos(2 * np.pi * u[1]), r0 * np.sin(2 * np.pi * u[1]), r1 * np.cos(2 * np.pi * u[3])], 1)
    return c.astype(np.float32)
