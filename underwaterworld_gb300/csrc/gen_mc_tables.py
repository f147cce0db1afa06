"""Generate ``mc_tables.h`` from the reference's marching-cubes tables.

The two tables (``EDGE_VERTEX_INDICES[12][2]`` and ``TRIANGULATION[256][16]``)
are parsed from ``underwater_world/src/marching_table.rs:1-273`` of
LelsersLasers/UnderwaterWorld (MIT licence, Copyright (c) 2024 Millan Kumar)
instead of being typed in, so the CUDA kernels and the CPU oracle use exactly
the rows the reference walks.  Two derived tables are added:

* ``UWW_CASE_NTRI[256]``  -- triangles per case (row length before -1, / 3);
* ``UWW_CASE_EDGES[256]`` -- 12-bit mask of the edges a case's row references;
* ``UWW_EDGE_BEFORE[256][12]`` -- per case and edge, the mask of the edges the
  row references for the first time before edge e's first reference, so a
  cell's k-th new vertex (in first-reference order) has rank
  popcount(owned & before[case][e]).

Usage: ``python gen_mc_tables.py <path to marching_table.rs> [out.h]``.
The generated header is committed; this script only runs when the tables
must be regenerated.
"""
import re
import sys
from pathlib import Path


def parse(src: str):
    m = re.search(r"EDGE_VERTEX_INDICES[^=]*=\s*\[(.*?)\];", src, re.S)
    edges = [tuple(int(v) for v in pair)
             for pair in re.findall(r"\[\s*(\d+)\s*,\s*(\d+)\s*\]", m.group(1))]
    m = re.search(r"TRIANGULATION[^=]*=\s*\[(.*)\];", src, re.S)
    rows = [[int(v) for v in row.split(",") if v.strip()]
            for row in re.findall(r"\[([-\d,\s]+)\]", m.group(1))]
    assert len(edges) == 12 and all(len(e) == 2 for e in edges)
    assert len(rows) == 256 and all(len(r) == 16 for r in rows)
    return edges, rows


def edge_owner(edges):
    """[oriented dedup?][x==0 | y==0 << 1 | z==0 << 2][e] -> the cell that creates
    the vertex of a cell's edge e: bits 0-3 its edge id e', bits 4/5/6 set when
    it lies one cell back in x/y/z.  Only earlier cells (offsets -1 or 0) can
    own an edge, so the low-side boundary flags decide."""
    share = edge_share(edges)
    out = []
    for oriented in (0, 1):
        row = []
        for f in range(8):
            lo = [bool(f & 1), bool(f & 2), bool(f & 4)]
            ents = []
            for e in range(12):
                for dx, dy, dz, e2, same in share[e]:
                    if oriented and not same:
                        continue
                    d = (dx, dy, dz)
                    if any(d[i] > 0 for i in range(3)):
                        continue
                    if any(d[i] < 0 and lo[i] for i in range(3)):
                        continue
                    ents.append(e2 | ((dx < 0) << 4) | ((dy < 0) << 5) | ((dz < 0) << 6))
                    break
                else:
                    raise AssertionError("every edge has an owner")
            row.append(ents)
        out.append(row)
    return out


def first_before(rows):
    out = []
    for r in rows:
        order = []
        for e in r:
            if e < 0:
                break
            if e not in order:
                order.append(e)
        masks = [0] * 12
        for i, e in enumerate(order):
            for f in order[:i]:
                masks[e] |= 1 << f
        out.append(masks)
    return out


def derive(rows):
    ntri, emask = [], []
    for r in rows:
        n = r.index(-1) if -1 in r else 16
        assert n % 3 == 0, "row length must be a multiple of 3"
        assert all(v == -1 for v in r[n:])
        ntri.append(n // 3)
        m = 0
        for e in r[:n]:
            m |= 1 << e
        emask.append(m)
    return ntri, emask


# Cube corner offsets in the reference's order (chunk.rs:144-153).
CORNERS = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1),
           (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]


def edge_share(edges):
    """For each cube edge e of a cell at the origin: the four cells that hold
    the same physical edge, as (dx, dy, dz, e', same_orientation), sorted in
    the builder's cell order (x outer, then y, then z)."""
    table = []
    for a, b in edges:
        A, B = CORNERS[a], CORNERS[b]
        axis = [i for i in range(3) if A[i] != B[i]][0]
        lo = tuple(min(A[i], B[i]) for i in range(3))
        others = [i for i in range(3) if i != axis]
        cands = []
        for du in (0, 1):
            for dv in (0, 1):
                C = list(lo)
                C[others[0]] -= du
                C[others[1]] -= dv
                C = tuple(C)
                found = None
                for e2, (a2, b2) in enumerate(edges):
                    A2 = tuple(CORNERS[a2][i] + C[i] for i in range(3))
                    B2 = tuple(CORNERS[b2][i] + C[i] for i in range(3))
                    if {A2, B2} == {A, B}:
                        found = (C[0], C[1], C[2], e2, int(A2 == A))
                assert found is not None
                cands.append(found)
        cands.sort(key=lambda t: (t[0], t[1], t[2]))
        table.append(cands)
    return table


def owned_masks(edges):
    """[oriented dedup?][boundary flags] -> mask of the edges a cell creates vertices for.

    Flag bits: 1 x==0, 2 y==0, 4 z==0, 8 x==N-1, 16 y==N-1, 32 z==N-1.  A cell
    owns edge e when no earlier cell (in stream order) inside the chunk holds
    the same edge (with the same orientation, for oriented dedup)."""
    share = edge_share(edges)
    out = []
    for oriented in (0, 1):
        row = []
        for f in range(64):
            lo = [bool(f & 1), bool(f & 2), bool(f & 4)]
            hi = [bool(f & 8), bool(f & 16), bool(f & 32)]
            m = 0
            for e in range(12):
                for dx, dy, dz, e2, same in share[e]:
                    if oriented and not same:
                        continue
                    d = (dx, dy, dz)
                    if any((d[i] < 0 and lo[i]) or (d[i] > 0 and hi[i]) for i in range(3)):
                        continue
                    if d == (0, 0, 0) and e2 == e:
                        m |= 1 << e
                    break
            row.append(m)
        out.append(row)
    return out  # index 0: one vertex per edge, 1: oriented (reference) dedup


def emit(edges, rows, ntri, emask) -> str:
    out = [
        "// Generated by gen_mc_tables.py from underwater_world/src/marching_table.rs:1-273",
        "// of LelsersLasers/UnderwaterWorld (MIT licence, Copyright (c) 2024 Millan Kumar).",
        "// Do not edit by hand; regenerate with the script.",
        "#pragma once",
        "#include <stdint.h>",
        "// UWW_TABLE_QUAL lets CUDA code place the tables in __constant__ memory.",
        "#ifndef UWW_TABLE_QUAL",
        "#define UWW_TABLE_QUAL",
        "#endif",
        "",
        "// Bourke cube-edge -> (corner a, corner b); marching_table.rs:1-14.",
        "UWW_TABLE_QUAL static const uint8_t UWW_EDGE_CORNERS[12][2] = {",
    ]
    out.append(",\n".join(f"    {{{a}, {b}}}" for a, b in edges))
    out += ["};", "",
            "// Bourke triangulation, -1 terminated; marching_table.rs:16-273.",
            "UWW_TABLE_QUAL static const int8_t UWW_TRI_TABLE[256][16] __attribute__((aligned(16))) = {"]
    out.append(",\n".join("    {" + ", ".join(f"{v:2d}" for v in r) + "}" for r in rows))
    out += ["};", "", "// Triangles per case (derived).",
            "UWW_TABLE_QUAL static const uint8_t UWW_CASE_NTRI[256] = {"]
    out.append(",\n".join("    " + ", ".join(str(v) for v in ntri[i:i + 16])
                          for i in range(0, 256, 16)))
    out += ["};", "", "// Edges referenced by each case's row, bit e = edge e (derived).",
            "UWW_TABLE_QUAL static const uint16_t UWW_CASE_EDGES[256] = {"]
    out.append(",\n".join("    " + ", ".join(f"0x{v:03x}" for v in emask[i:i + 8])
                          for i in range(0, 256, 8)))
    out += ["};", "",
            "// For cube edge e: the 4 cells sharing that edge as {dx, dy, dz, e', same orientation},",
            "// in cell order (x outer, y, z inner).  The first one inside the chunk (and, for",
            "// oriented dedup, with the same orientation) is where the reference creates the vertex.",
            "UWW_TABLE_QUAL static const int8_t UWW_EDGE_SHARE[12][4][5] = {"]
    rows_out = []
    for e, cands in enumerate(edge_share(edges)):
        rows_out.append("    {" + ", ".join("{%d, %d, %d, %d, %d}" % c for c in cands) + "}")
    out.append(",\n".join(rows_out))
    out += ["};", "",
            "// Owned-edge mask of a cell by its boundary flags (bit 1 x==0, 2 y==0, 4 z==0, 8 x==N-1,",
            "// 16 y==N-1, 32 z==N-1): [0] one vertex per edge, [1] oriented (reference) dedup; derived from UWW_EDGE_SHARE.",
            "UWW_TABLE_QUAL static const uint16_t UWW_OWNED_MASK[2][64] = {"]
    om = owned_masks(edges)
    out.append(",\n".join("    {" + ", ".join(f"0x{v:03x}" for v in r) + "}" for r in om))
    out += ["};", "",
            "// Owner of a cell's edge e by [oriented dedup][x==0 | y==0 << 1 | z==0 << 2]: bits 0-3 the",
            "// owner's edge id, bits 4/5/6 the owner one cell back in x/y/z (derived from UWW_EDGE_SHARE).",
            "UWW_TABLE_QUAL static const uint8_t UWW_EDGE_OWNER[2][8][12] = {"]
    own = edge_owner(edges)
    out.append(",\n".join("    {" + ", ".join("{" + ", ".join(f"0x{v:02x}" for v in r) + "}" for r in m) + "}"
                          for m in own))
    out += ["};", "",
            "// Per case and edge e: mask of the edges the row references for the first time before",
            "// e's first reference (derived).  A cell numbers the vertices of its owned edges in",
            "// first-reference order, so edge e's vertex is popcount(owned & before[case][e]).",
            "UWW_TABLE_QUAL static const uint16_t UWW_EDGE_BEFORE[256][12] __attribute__((aligned(16))) = {"]
    out.append(",\n".join("    {" + ", ".join(f"0x{v:03x}" for v in r) + "}" for r in first_before(rows)))
    out += ["};", ""]
    return "\n".join(out)


def main(argv):
    src = Path(argv[1]).read_text()
    dst = Path(argv[2]) if len(argv) > 2 else Path(__file__).with_name("mc_tables.h")
    edges, rows = parse(src)
    ntri, emask = derive(rows)
    dst.write_text(emit(edges, rows, ntri, emask))
    print(f"wrote {dst}")


if __name__ == "__main__":
    main(sys.argv)
