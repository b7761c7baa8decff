"""Generate mc_tables.h: the Marching Cubes case tables in this library's packed encoding.

Two tables follow from the case rules and are computed here:
  * edge mask per case: the edges whose end vertices lie on different sides of the isovalue
    (same content as e_pattern in mc/MarchingCubes.h);
  * ambiguity per case: a face whose diagonal corners share a side, or a body-diagonal pair of
    lone corners (same content as t_ambig in mc/MarchingCubes.h and cpp_dmc/LookupTables.h,
    where the value 105 marks the ambiguous cases).

Two tables are arbitrary data and are taken from the reference's tables via the golden fixture
tests/golden/ref_tables.json:
  * the start edge of the single contour of every unambiguous case (the contour itself follows
    from the face rules; only its starting edge is a free choice in cpp_dmc/LookupTables.h
    r_pattern), packed as one nibble per case;
  * the triangle list of every unambiguous case (mc/MarchingCubes.h t_pattern), packed as a
    64-bit word: bits 0-3 the triangle count, then 4-bit edge ids, three per triangle.

Run:  python tmc_gb300/csrc/gen_tables.py   (rewrites tmc_gb300/csrc/mc_tables.h)
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# Cell topology (vertex v = (v&1, v>>1&1, v>>2&1)); edge endpoints.
EDGE_V = [(0, 1), (1, 3), (2, 3), (0, 2), (4, 5), (5, 7), (6, 7), (4, 6), (0, 4), (1, 5), (3, 7), (2, 6)]
# Faces seen from outside: oriented vertex quadruple and edge quadruple.
FACE_V = [(0, 2, 1, 3), (5, 7, 4, 6), (4, 0, 5, 1), (2, 6, 3, 7), (4, 6, 0, 2), (1, 3, 5, 7)]
FACE_E = [(3, 2, 1, 0), (5, 6, 7, 4), (8, 0, 9, 4), (11, 6, 10, 2), (7, 11, 3, 8), (1, 10, 5, 9)]


def edge_mask(c: int) -> int:
    m = 0
    for e, (a, b) in enumerate(EDGE_V):
        if ((c >> a) & 1) != ((c >> b) & 1):
            m |= 1 << e
    return m


def face_case(c: int, f: int) -> int:
    v0, v1, v2, v3 = FACE_V[f]
    return ((c >> v0) & 1) | ((c >> v1) & 1) << 1 | ((c >> v2) & 1) << 2 | ((c >> v3) & 1) << 3


def ambiguous(c: int) -> bool:
    if any(face_case(c, f) in (6, 9) for f in range(6)):
        return True
    for s in (c, (~c) & 255):
        if bin(s).count("1") == 2:
            a, b = [v for v in range(8) if (s >> v) & 1]
            if a ^ b == 7:
                return True
    return False


def face_segments(c: int):
    """Oriented segments on the faces of an unambiguous case: edge -> next edge."""
    to = {}
    rules = {1: [(0, 3)], 2: [(1, 0)], 3: [(1, 3)], 4: [(3, 2)], 5: [(0, 2)], 7: [(1, 2)], 8: [(2, 1)],
             10: [(2, 0)], 11: [(2, 3)], 12: [(3, 1)], 13: [(0, 1)], 14: [(3, 0)]}
    for f in range(6):
        fe = FACE_E[f]
        for a, b in rules.get(face_case(c, f), []):
            to[fe[a]] = fe[b]
    return to


def contours(c: int):
    to = dict(face_segments(c))
    out = []
    for e in range(12):
        if e in to:
            cnt = [e]
            nxt = to[e]
            while nxt != e:
                cnt.append(nxt)
                nxt = to.pop(nxt)
            to.pop(e, None)
            out.append(cnt)
    return out


def main():
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "ref_tables.json")))
    rp, tp = ref["dmc_r_pattern"], ref["mc_t_pattern"]
    e_pat = [edge_mask(c) for c in range(256)]
    amb = [ambiguous(c) for c in range(256)]
    start = []
    for c in range(256):
        row = rp[17 * c: 17 * c + 17]
        if amb[c] or row[0] == 0:
            start.append(15)
            continue
        assert row[0] == 1
        mine = contours(c)
        assert len(mine) == 1 and sorted(mine[0]) == sorted(row[2: 2 + row[1]])
        start.append(row[2])
    tris = []
    for c in range(256):
        row = [x for x in tp[16 * c: 16 * c + 16]]
        n = 0
        word = 0
        for t in range(0, 15, 3):
            if row[t] == -1:
                break
            for k in range(3):
                word |= (row[t + k] & 0xF) << (4 + 4 * (3 * n + k))
            n += 1
        tris.append(word | n)
    amb_words = [0, 0, 0, 0]
    for c in range(256):
        if amb[c]:
            amb_words[c >> 6] |= 1 << (c & 63)
    L = []
    L.append("// Generated by tmc_gb300/csrc/gen_tables.py -- do not edit.")
    L.append("// Marching Cubes case tables in this library's packed encoding (see the generator).")
    L.append("#pragma once")
    L.append("#include <stdint.h>")
    L.append("")
    L.append("// Edges crossed by the isosurface, per case (bit e = edge e).")
    L.append("#define TMC_EDGE_MASK_INIT { \\")
    for r in range(0, 256, 16):
        L.append("  " + ", ".join(str(x) for x in e_pat[r:r + 16]) + ", \\")
    L.append("}")
    L.append("static const uint16_t TMC_EDGE_MASK[256] = TMC_EDGE_MASK_INIT;")
    L.append("// Ambiguous cases (bit c of word c/64).")
    for i, w in enumerate(amb_words):
        L.append(f"#define TMC_AMBIGUOUS_W{i} 0x{w:016x}ull")
    L.append("static const uint64_t TMC_AMBIGUOUS[4] = {TMC_AMBIGUOUS_W0, TMC_AMBIGUOUS_W1, TMC_AMBIGUOUS_W2, TMC_AMBIGUOUS_W3};")
    L.append("// Start edge of the single contour of each unambiguous case, two cases per byte")
    L.append("// (low nibble = even case); 15 = no contour / ambiguous case.")
    packed = [start[2 * i] | (start[2 * i + 1] << 4) for i in range(128)]
    L.append("static const uint8_t TMC_CONTOUR_START[128] = {")
    for r in range(0, 128, 16):
        L.append("  " + ", ".join(str(x) for x in packed[r:r + 16]) + ",")
    L.append("};")
    L.append("// Triangles of each unambiguous case: bits 0-3 count, then 4-bit edge ids (3 per triangle).")
    L.append("#define TMC_TRIANGLES_INIT { \\")
    for r in range(0, 256, 4):
        L.append("  " + ", ".join(f"0x{w:016x}ull" for w in tris[r:r + 4]) + ", \\")
    L.append("}")
    L.append("static const uint64_t TMC_TRIANGLES[256] = TMC_TRIANGLES_INIT;")
    # ---- packed topology (4 bits per entry) and the per-case contour of unambiguous cases ----
    def pack(vals):
        w = 0
        for i, x in enumerate(vals):
            assert 0 <= x < 16
            w |= x << (4 * i)
        return w
    EDGE_GLOBAL = [(0, 0, 0, 0), (1, 0, 0, 1), (0, 1, 0, 0), (0, 0, 0, 1), (0, 0, 1, 0), (1, 0, 1, 1),
                   (0, 1, 1, 0), (0, 0, 1, 1), (0, 0, 0, 2), (1, 0, 0, 2), (1, 1, 0, 2), (0, 1, 0, 2)]
    QUAD_SLOT = [(0, 0), (0, 0), (3, 1), (3, 1), (1, 3), (1, 3), (2, 2), (2, 2), (0, 0), (3, 1), (2, 2), (1, 3)]
    L.append("")
    L.append("// Packed cell topology, 4 bits per entry (entry i at bits 4i..4i+3).")
    L.append(f"#define TMC_PK_EDGE_V0 0x{pack([a for a, b in EDGE_V]):012x}ull   // first end vertex of edge e")
    L.append(f"#define TMC_PK_EDGE_V1 0x{pack([b for a, b in EDGE_V]):012x}ull   // second end vertex of edge e")
    L.append(f"#define TMC_PK_EDGE_OFF 0x{pack([g[0] | g[1] << 1 | g[2] << 2 for g in EDGE_GLOBAL]):012x}ull  // lower grid point offset (di|dj<<1|dk<<2)")
    L.append(f"#define TMC_PK_EDGE_AXIS 0x{pack([g[3] for g in EDGE_GLOBAL]):012x}ull // axis of edge e")
    L.append(f"#define TMC_PK_QUAD_SLOT0 0x{pack([q[0] for q in QUAD_SLOT]):012x}ull // quad slot, first end vertex >= iso")
    L.append(f"#define TMC_PK_QUAD_SLOT1 0x{pack([q[1] for q in QUAD_SLOT]):012x}ull // quad slot, first end vertex < iso")
    for f in range(6):
        L.append(f"#define TMC_PK_FACE_V{f} 0x{pack(FACE_V[f]):04x}u")
        L.append(f"#define TMC_PK_FACE_E{f} 0x{pack(FACE_E[f]):04x}u")
    L.append("// The contour of each unambiguous case, rotated to the start edge above: bits 0-3 size,")
    L.append("// then the edges, one nibble each.  0 for ambiguous and empty cases.")
    L.append("#define TMC_CASE_CONTOUR_INIT { \\")
    words = []
    for c in range(256):
        if amb[c] or start[c] == 15:
            words.append(0)
            continue
        cnt = contours(c)[0]
        r = cnt.index(start[c])
        cnt = cnt[r:] + cnt[:r]
        words.append(pack([len(cnt)] + cnt))
    for r in range(0, 256, 4):
        L.append("  " + ", ".join(f"0x{w:016x}ull" for w in words[r:r + 4]) + ", \\")
    L.append("}")
    L.append("static const uint64_t TMC_CASE_CONTOUR[256] = TMC_CASE_CONTOUR_INIT;")
    with open(os.path.join(HERE, "mc_tables.h"), "w") as f:
        f.write("\n".join(L) + "\n")


if __name__ == "__main__":
    main()
