"""A second, independent restatement of the noise in pure Python, checked
against the oracle's C restatement.

The noise lives in the un-vendored crate `noise` 0.8.2 (called at
underwater_world/src/perlin_util.rs:13; seeded at state.rs:359).  This file
restates its published algorithm a second time, in a different form from the
oracle.
* The seeded permutation: XorShift128 (x = 1, y = z = w = seed), then rand
  0.8's Fisher-Yates shuffle with the widening-multiply bounded draw.
* `perlin_3d`: the hash P[P[P[x] ^ y] ^ z], the 16-entry gradient table, the
  quintic fade, and nested linear interpolation (the oracle uses the
  k-polynomial form), scaled by 2/sqrt(3).
* `perlin_3d_octaves` and `iso_at` (perlin_util.rs:6-29), in reference
  semantics: f64 noise cast to f32, then the f32 terraced bias.
No GPU is needed.
"""
import math

import numpy as np

from underwaterworld_gb300 import abi

M32 = 0xFFFFFFFF


def seeded_perm(seed: int) -> list[int]:
    x, y, z, w = 1, seed & M32, seed & M32, seed & M32

    def next_u32():
        nonlocal x, y, z, w
        t = (x ^ (x << 11)) & M32
        x, y, z = y, z, w
        w = (w ^ (w >> 19) ^ t ^ (t >> 8)) & M32
        return w

    def below(n):
        # rand 0.8 UniformInt<u32>::sample_single: accept the low word of
        # v * n when it is at most (n << leading_zeros(n)) - 1
        zone = ((n << (32 - n.bit_length())) & M32) - 1
        while True:
            m = next_u32() * n
            if (m & M32) <= zone:
                return m >> 32

    p = list(range(256))
    for i in range(255, 0, -1):
        j = below(i + 1)
        p[i], p[j] = p[j], p[i]
    return p


GRAD = [(1, 1, 0), (-1, 1, 0), (1, -1, 0), (-1, -1, 0), (1, 0, 1), (-1, 0, 1), (1, 0, -1), (-1, 0, -1),
        (0, 1, 1), (0, -1, 1), (0, 1, -1), (0, -1, -1), (1, 1, 0), (-1, 1, 0), (0, -1, 1), (0, -1, -1)]


def perlin(P, px: float, py: float, pz: float) -> float:
    ix, iy, iz = math.floor(px), math.floor(py), math.floor(pz)
    dx, dy, dz = px - ix, py - iy, pz - iz

    def corner(i, j, k):
        h = P[P[P[(ix + i) & 255] ^ ((iy + j) & 255)] ^ ((iz + k) & 255)]
        g = GRAD[h & 15]
        return g[0] * (dx - i) + g[1] * (dy - j) + g[2] * (dz - k)

    def fade(t):
        return t * t * t * (t * (t * 6 - 15) + 10)

    def lerp(t, a, b):
        return a + t * (b - a)

    a, b, c = fade(dx), fade(dy), fade(dz)
    x00 = lerp(a, corner(0, 0, 0), corner(1, 0, 0))
    x10 = lerp(a, corner(0, 1, 0), corner(1, 1, 0))
    x01 = lerp(a, corner(0, 0, 1), corner(1, 0, 1))
    x11 = lerp(a, corner(0, 1, 1), corner(1, 1, 1))
    return lerp(c, lerp(b, x00, x10), lerp(b, x01, x11)) * (2.0 / math.sqrt(3.0))


def iso_at_world(P, p: abi.Params, wx: float, wy: float, wz: float) -> np.float32:
    """Reference-semantics density at a world point, reference parameters
    (terraced bias, normalised fBm)."""
    f32 = np.float32
    bf = float(f32(p.base_freq))
    nx, ny, nz = wx * bf, wy * bf, wz * bf
    total, amp_sum, m, a = 0.0, 0.0, 1.0, float(f32(p.amplitude))
    for _ in range(p.octaves):
        total += perlin(P, nx * m, ny * m, nz * m) * a
        amp_sum += a
        m *= float(f32(p.lacunarity))
        a *= float(f32(p.persistence))
    f = f32(total / amp_sum)
    adj = f32(f32(nz) * f32(p.bias_a)) / f32(p.bias_b)
    return f32(f32(adj + f) - np.fmod(adj, f32(p.bias_c)))


def test_seeded_permutation_matches_the_product_and_the_oracle(oracle):
    for seed in (0, 1, 7, 12345, 0xFFFFFFFF):
        want = seeded_perm(seed)
        assert sorted(want) == list(range(256))
        assert list(abi.perm_table(seed)) == want, seed
        assert list(oracle.perm(seed)) == want, seed


def test_perlin_matches_the_oracle(oracle):
    rng = np.random.default_rng(11)
    pts = np.concatenate([rng.uniform(-300, 300, (300, 3)), rng.integers(-40, 40, (20, 3)) + 0.5,
                          rng.integers(-40, 40, (20, 3)).astype(np.float64)])
    for seed in (0, 3):
        P = seeded_perm(seed)
        want = np.array([perlin(P, *pt) for pt in pts])
        got = oracle.perlin(seed, pts)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
        assert np.abs(want[-20:]).max() == 0.0  # zero at lattice points


def test_reference_density_matches_the_oracle(oracle):
    p = abi.reference_params()
    P = seeded_perm(p.seed)
    rng = np.random.default_rng(5)
    xyz = rng.uniform(-64, 64, (400, 3)).astype(np.float32)
    want = np.array([iso_at_world(P, p, *map(float, pt)) for pt in xyz], dtype=np.float32)
    got = oracle.density_at(p, xyz, precision=oracle.F64)
    # the Perlin values differ from the oracle's in the last f64 bits at most
    # (lerp form against k-polynomial), far below one f32 step: equal after the cast
    np.testing.assert_array_equal(got, want)
