"""Generate tests/golden/mc_known_answers.npz.

Known-answer vectors for the marching-cubes stage, computed by a pure-Python
restatement of Chunk::build_mesh (underwater_world/src/chunk.rs:135-264) that
reads the triangulation straight from the reference's
underwater_world/src/marching_table.rs (not from the generated C header), in
numpy float32 scalar arithmetic (one rounding per operation, like the
reference's f32 code).  Colours use numpy's float32 power and are compared to
a tolerance by the tests.

Cases (each a list of chunks with caller-provided samples):
  * single_cell: all 256 cases of one cell, corner samples -1 (inside) / +1,
    iso-level 0, so every vertex sits at an edge midpoint;
  * single_cell_random: all 256 cases with random magnitudes, iso-level 0;
  * grids: 2^3- and 3^3-cell chunks of random samples at the reference
    iso-level -0.1, at several chunk positions.

Run from the repository root (needs the reference checkout):
    python tests/golden/make_golden.py /path/to/UnderwaterWorld
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

f32 = np.float32
CORNERS = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]
CHUNK_SIZE = 16
ISO_REF = f32(-0.1)


def parse_tables(path: Path):
    src = path.read_text()
    m = re.search(r"EDGE_VERTEX_INDICES[^=]*=\s*\[(.*?)\];", src, re.S)
    edges = [(int(a), int(b)) for a, b in re.findall(r"\[\s*(\d+)\s*,\s*(\d+)\s*\]", m.group(1))]
    m = re.search(r"TRIANGULATION[^=]*=\s*\[(.*)\];", src, re.S)
    rows = [[int(v) for v in r.split(",") if v.strip()] for r in re.findall(r"\[([-\d,\s]+)\]", m.group(1))]
    return edges, rows


def hsv_to_rgb(hue, sat, val):
    r0 = f32(np.fmod(hue, f32(360.0)))
    hue = f32(r0 + f32(360.0)) if r0 < 0 else r0
    c = f32(val * sat)
    h = f32(hue / f32(60.0))
    x = f32(c * f32(f32(1.0) - abs(f32(f32(np.fmod(h, f32(2.0))) - f32(1.0)))))
    m = f32(val - c)
    z = f32(0.0)
    if 0 <= h < 1:
        r, g, b = c, x, z
    elif 1 <= h < 2:
        r, g, b = x, c, z
    elif 2 <= h < 3:
        r, g, b = z, c, x
    elif 3 <= h < 4:
        r, g, b = z, x, c
    elif 4 <= h < 5:
        r, g, b = x, z, c
    else:
        r, g, b = c, z, x
    return [f32(f32(r + m) * f32(255.0)), f32(f32(g + m) * f32(255.0)), f32(f32(b + m) * f32(255.0))]


def to_srgb(c):
    return [f32(np.power(f32(f32(f32(v / f32(255.0)) + f32(0.055)) / f32(1.055)), f32(2.4))) for v in c]


def build_mesh(edges, rows, isos, N, pos, iso_level):
    """chunk.rs:135-264 for one chunk of N cells; isos indexed (x*S + y)*S + z."""
    S = N + 1
    s = f32(f32(CHUNK_SIZE) / f32(N))
    off = [p * CHUNK_SIZE for p in pos]
    verts, colors, keys, inds, cases = [], [], [], [], []
    for x in range(N):
        for y in range(N):
            for z in range(N):
                cc = [(x + a, y + b, z + c) for a, b, c in CORNERS]
                case = 0
                for i, (a, b, c) in enumerate(cc):
                    if isos[(a * S + b) * S + c] < iso_level:
                        case |= 1 << i
                cases.append(case)
                for e in rows[case]:
                    if e == -1:
                        break
                    ca, cb = edges[e]
                    A, B = cc[ca], cc[cb]
                    key = (A, B)
                    if key in keys:
                        inds.append(keys.index(key))
                        continue
                    sa = [f32(f32(v) * s) for v in A]
                    sb = [f32(f32(v) * s) for v in B]
                    ia = isos[(A[0] * S + A[1]) * S + A[2]]
                    ib = isos[(B[0] * S + B[1]) * S + B[2]]
                    t = f32(f32(iso_level - ia) / f32(ib - ia))
                    mid = [f32(sa[k] + f32(t * f32(sb[k] - sa[k]))) for k in range(3)]
                    wz = f32(mid[2] + f32(off[2]))
                    ratio = f32(wz / f32(CHUNK_SIZE))
                    mix = f32(f32(ratio - f32(-2.0)) / f32(f32(2.0) - f32(-2.0)))
                    vi = f32(f32(cb % 3) / f32(9.0))
                    hue = f32(f32(-150.0) + f32(f32(210.0) * mix))
                    col = to_srgb(hsv_to_rgb(hue, f32(0.6), f32(f32(0.4) + vi)))
                    keys.append(key)
                    verts.append([f32(mid[0] + f32(off[0])), f32(mid[1] + f32(off[1])), wz])
                    colors.append(col)
                    inds.append(len(keys) - 1)
    return (np.array(verts, np.float32).reshape(-1, 3), np.array(colors, np.float32).reshape(-1, 3),
            np.array(inds, np.uint32), np.array(cases, np.uint8))


def make_case_set(edges, rows, chunks, iso_level):
    """chunks: list of (N, pos, isos f32 array)."""
    out = {"cells": [], "pos": [], "samples": [], "verts": [], "colors": [], "inds": [], "cases": [],
           "num_verts": [], "num_inds": []}
    for N, pos, isos in chunks:
        v, c, i, cs = build_mesh(edges, rows, isos, N, pos, iso_level)
        out["cells"].append(N)
        out["pos"].append(pos)
        out["samples"].append(isos)
        out["verts"].append(v)
        out["colors"].append(c)
        out["inds"].append(i)
        out["cases"].append(cs)
        out["num_verts"].append(len(v))
        out["num_inds"].append(len(i))
    return {
        "cells": np.array(out["cells"], np.uint32), "pos": np.array(out["pos"], np.int32),
        "samples": np.concatenate(out["samples"]).astype(np.float32),
        "verts": np.concatenate(out["verts"]), "colors": np.concatenate(out["colors"]),
        "inds": np.concatenate(out["inds"]), "cases": np.concatenate(out["cases"]),
        "num_verts": np.array(out["num_verts"], np.uint32), "num_inds": np.array(out["num_inds"], np.uint32),
        "iso_level": np.float32(iso_level),
    }


def corner_grid(case, values):
    """2x2x2 samples for one cell: corner i gets -|v_i| if bit i of case is set, else +|v_i|."""
    g = np.zeros(8, np.float32)
    for i, (a, b, c) in enumerate(CORNERS):
        v = abs(values[i])
        g[(a * 2 + b) * 2 + c] = -v if (case >> i) & 1 else v
    return g


def main(ref_root: str):
    edges, rows = parse_tables(Path(ref_root) / "underwater_world" / "src" / "marching_table.rs")
    rng = np.random.default_rng(20240603)
    sets = {}
    sets["single_cell"] = make_case_set(
        edges, rows, [(1, (0, 0, 0), corner_grid(c, [1.0] * 8)) for c in range(256)], f32(0.0))
    sets["single_cell_random"] = make_case_set(
        edges, rows, [(1, (c % 5 - 2, c % 3 - 1, c % 4 - 2), corner_grid(c, rng.uniform(0.05, 2.0, 8)))
                      for c in range(256)], f32(0.0))
    grids = []
    for k in range(12):
        N = 2 if k < 8 else 3
        pos = tuple(int(v) for v in rng.integers(-3, 4, 3))
        isos = rng.normal(0.0, 0.5, (N + 1) ** 3).astype(np.float32)
        grids.append((N, pos, isos))
    sets["grids"] = make_case_set(edges, rows, grids, ISO_REF)
    flat = {f"{name}/{k}": v for name, d in sets.items() for k, v in d.items()}
    dst = Path(__file__).with_name("mc_known_answers.npz")
    np.savez_compressed(dst, **flat)
    print(f"wrote {dst}: " + ", ".join(f"{n}: {len(d['cells'])} chunks, {int(d['num_inds'].sum())} inds"
                                      for n, d in sets.items()))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <UnderwaterWorld checkout>")
    main(sys.argv[1])
