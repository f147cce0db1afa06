"""A second, independent restatement of the vertex colour ramp in numpy
float32, checked against the oracle's colours.

The ramp is chunk.rs:215-222: the world z in chunks is mixed between
world::MIN_Z = -2 and MAX_Z = 2 (util.rs:93-95).  That gives a hue from
MIN_HUE = -150 to MAX_HUE = 60, and a value of BASE_VALUE = 0.4 plus
(corner_b % 3) / 9.  Then come hsv_to_rgb (util.rs:122-153) and to_srgb
(util.rs:106-112).  A vertex's corner index is not part of the output, so each
vertex's colour must equal, bit for bit, one of the three candidates of its
z.  No GPU is needed.
"""
import ctypes
import ctypes.util

import numpy as np

from underwaterworld_gb300 import abi, workloads

f32 = np.float32

# the C library's powf, as Rust's f32::powf and the oracle call it (numpy's own
# float32 power may round differently in the last bit)
_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.powf.restype = ctypes.c_float
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]


def rem_euclid(a, b):
    r = np.fmod(a, b)
    return r + abs(b) if r < 0 else r


def hsv_to_rgb(hue, saturation, value):
    hue = rem_euclid(f32(hue), f32(360))
    c = f32(value * saturation)
    h = f32(hue / f32(60))
    x = f32(c * f32(f32(1) - abs(f32(np.fmod(h, f32(2)) - f32(1)))))
    m = f32(value - c)
    z = f32(0)
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
    return [f32(f32(v + m) * f32(255)) for v in (r, g, b)]


def to_srgb(rgb):
    return [f32(_libm.powf(float(f32(f32(f32(v / f32(255)) + f32(0.055)) / f32(1.055))), 2.4)) for v in rgb]


def colour_candidates(world_z):
    ratio = f32(f32(f32(world_z / f32(16)) - f32(-2)) / f32(f32(2) - f32(-2)))
    hue = f32(f32(-150) + f32(f32(f32(60) - f32(-150)) * ratio))
    return [to_srgb(hsv_to_rgb(hue, f32(0.6), f32(f32(0.4) + f32(f32(k) / f32(9))))) for k in range(3)]


def test_vertex_colours_follow_the_ramp(oracle):
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_COLOR)
    b = oracle.build_chunks(p, d[::3], precision=oracle.F64)
    verts = b.verts
    assert len(verts) > 1000
    used = set()
    for v in verts:
        cands = colour_candidates(f32(v["pos"][2]))
        got = [f32(c) for c in v["color"]]
        hits = [k for k, c in enumerate(cands) if all(f32(g) == f32(w) for g, w in zip(got, c))]
        assert hits, (v, cands)
        used.update(hits)
    assert used == {0, 1, 2}
