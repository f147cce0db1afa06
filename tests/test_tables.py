"""Invariants of the marching-cubes tables generated from marching_table.rs."""
import re
from pathlib import Path

import numpy as np

HDR = Path(__file__).resolve().parent.parent / "underwaterworld_gb300" / "csrc" / "mc_tables.h"
CORNERS = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]


def _array(name):
    src = HDR.read_text()
    m = re.search(name + r"\[[^=]*=\s*\{(.*?)\};", src, re.S)
    return [int(v, 0) for v in re.findall(r"-?(?:0x[0-9a-f]+|\d+)", m.group(1))]


def tables():
    edges = np.array(_array("UWW_EDGE_CORNERS"), dtype=int).reshape(12, 2)
    tri = np.array(_array("UWW_TRI_TABLE"), dtype=int).reshape(256, 16)
    ntri = np.array(_array("UWW_CASE_NTRI"), dtype=int)
    emask = np.array(_array("UWW_CASE_EDGES"), dtype=int)
    share = np.array(_array("UWW_EDGE_SHARE"), dtype=int).reshape(12, 4, 5)
    return edges, tri, ntri, emask, share


def test_rows_are_whole_triangles_and_terminated():
    _, tri, ntri, _, _ = tables()
    for c in range(256):
        row = list(tri[c])
        n = row.index(-1) if -1 in row else 16
        assert n % 3 == 0 and n == 3 * ntri[c]
        assert all(v == -1 for v in row[n:])
        assert all(0 <= v < 12 for v in row[:n])


def test_empty_and_full_cases():
    _, tri, ntri, _, _ = tables()
    assert ntri[0] == 0 and ntri[255] == 0
    assert tri[0][0] == -1 and tri[255][0] == -1
    assert ntri.max() == 5


def test_each_row_uses_exactly_the_crossed_edges():
    """A crossed edge is used by every cell holding it: the basis of owner-cell dedup."""
    edges, _, _, emask, _ = tables()
    for c in range(256):
        crossed = 0
        for e, (a, b) in enumerate(edges):
            if ((c >> a) & 1) != ((c >> b) & 1):
                crossed |= 1 << e
        assert crossed == emask[c], c


def test_complement_cases_use_same_edges():
    _, _, ntri, emask, _ = tables()
    for c in range(256):
        assert emask[c] == emask[255 - c]


def test_edge_share_table():
    edges, _, _, _, share = tables()
    for e, (a, b) in enumerate(edges):
        A, B = np.array(CORNERS[a]), np.array(CORNERS[b])
        seen_self = False
        for dx, dy, dz, e2, same in share[e]:
            off = np.array([dx, dy, dz])
            a2, b2 = edges[e2]
            A2, B2 = np.array(CORNERS[a2]) + off, np.array(CORNERS[b2]) + off
            assert {tuple(A2), tuple(B2)} == {tuple(A), tuple(B)}
            assert bool(same) == (tuple(A2) == tuple(A))
            seen_self |= (dx, dy, dz, e2) == (0, 0, 0, e)
        assert seen_self
        keys = [tuple(s[:3]) for s in share[e]]
        assert keys == sorted(keys), "candidates must be in cell order"


def test_edge_before_is_first_reference_order():
    """UWW_EDGE_BEFORE[c][e] = edges first referenced before e's first reference,
    so popcount(owned & before) is the rank of e's vertex among a cell's new ones."""
    _, tri, ntri, emask, _ = tables()
    before = np.array(_array("UWW_EDGE_BEFORE"), dtype=int).reshape(256, 12)
    rng = np.random.default_rng(0)
    for c in range(256):
        row = [int(v) for v in tri[c][:3 * ntri[c]]]
        order = list(dict.fromkeys(row))
        for e in range(12):
            want = sum(1 << f for f in order[:order.index(e)]) if e in order else 0
            assert before[c][e] == want, (c, e)
        # rank of an edge among owned edges == position among owned first references
        for _ in range(4):
            owned = int(rng.integers(0, 1 << 12))
            seen = [e for e in order if owned >> e & 1]
            for k, e in enumerate(seen):
                assert bin(owned & before[c][e]).count("1") == k


def test_edge_owner_matches_first_sharing_cell():
    """UWW_EDGE_OWNER[oriented][low flags][e] names the first cell in stream order
    (inside the chunk, same orientation for oriented dedup) that holds edge e."""
    _, _, _, _, share = tables()
    owner = np.array(_array("UWW_EDGE_OWNER"), dtype=int).reshape(2, 8, 12)
    for oriented in (0, 1):
        for f in range(8):
            lo = [bool(f & 1), bool(f & 2), bool(f & 4)]
            for e in range(12):
                want = None
                for dx, dy, dz, e2, same in share[e]:
                    if oriented and not same:
                        continue
                    d = (dx, dy, dz)
                    if any((d[i] < 0 and lo[i]) for i in range(3)):
                        continue
                    want = (d, e2)
                    break
                o = owner[oriented][f][e]
                got = ((-((o >> 4) & 1), -((o >> 5) & 1), -((o >> 6) & 1)), o & 15)
                assert got == want, (oriented, f, e, got, want)
