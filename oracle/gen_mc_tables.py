"""Generate the packed marching-cubes triangle table used by the oracle and the
CUDA mesher from the reference's table (include/meshing/MarchingCubesTables.h:70).

The triangle list has to be the reference's own, row for row and in order: the
welded index buffer is defined by the order in which triangles are emitted. Each
row is stored here as one 64-bit word: up to 15 edge ids (0-11) as 4-bit nibbles,
least significant first, terminated by the nibble 0xF. The edge mask of a row is
not tabulated at all: it is computed from the cube index (an edge crosses when
its two corner bits differ), and this script checks that the reference's
edge_table equals that computation for all 256 rows.

Run once where the reference checkout is:
    python oracle/gen_mc_tables.py <reference>/include/meshing/MarchingCubesTables.h
Writes oracle/orc_mc_tables.h and azu_gb300/csrc/mc_tables.h.
"""
import os
import re
import sys

EDGE_CORNERS = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4),
                (0, 4), (1, 5), (2, 6), (3, 7)]


def crossing_mask(ci):
    m = 0
    for e, (a, b) in enumerate(EDGE_CORNERS):
        if ((ci >> a) & 1) != ((ci >> b) & 1):
            m |= 1 << e
    return m


def parse(text):
    et = re.search(r"edge_table\[256\]\s*=\s*\{(.*?)\};", text, re.S).group(1)
    edge = [int(v, 16) for v in re.findall(r"0x[0-9a-fA-F]+", et)]
    tt = re.search(r"tri_table\[256\]\[16\]\s*=\s*\{(.*)\};", text, re.S).group(1)
    rows = re.findall(r"\{([^{}]*)\}", tt)
    tri = [[int(v) for v in r.split(",")] for r in rows]
    assert len(edge) == 256 and len(tri) == 256 and all(len(r) == 16 for r in tri)
    return edge, tri


def pack(row):
    word, n = 0, 0
    for v in row:
        if v < 0:
            break
        word |= v << (4 * n)
        n += 1
    assert n % 3 == 0 and n <= 15
    word |= 0xF << (4 * n) if n < 16 else 0
    return word


def emit(words, guard, ns):
    lines = [
        "// Generated by oracle/gen_mc_tables.py from the reference's marching-cubes",
        "// triangle table. Row i = cube index i; edge ids (0-11) packed as 4-bit nibbles,",
        "// least significant first, terminated by 0xF. Do not edit by hand.",
        "#pragma once",
        "#include <stdint.h>",
        f"namespace {ns} {{",
        "static const uint64_t kTriRows[256] = {",
    ]
    for i in range(0, 256, 4):
        lines.append("    " + ", ".join(f"0x{w:016x}ull" for w in words[i:i + 4]) + ",")
    lines += ["};", f"}}  // namespace {ns}", ""]
    return "\n".join(lines)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: gen_mc_tables.py <path of the reference's include/meshing/MarchingCubesTables.h>")
    here = os.path.dirname(os.path.abspath(__file__))
    edge, tri = parse(open(sys.argv[1]).read())
    bad = [i for i in range(256) if edge[i] != crossing_mask(i)]
    if bad:
        sys.exit(f"reference edge_table differs from the crossing-edge rule at rows {bad}")
    for i, row in enumerate(tri):
        for v in row:
            if v >= 0 and not (crossing_mask(i) >> v) & 1:
                sys.exit(f"row {i} uses non-crossing edge {v}")
    words = [pack(r) for r in tri]
    with open(os.path.join(here, "orc_mc_tables.h"), "w") as f:
        f.write(emit(words, "ORC_MC_TABLES_H", "orc_tables"))
    with open(os.path.join(here, "..", "azu_gb300", "csrc", "mc_tables.h"), "w") as f:
        f.write(emit(words, "AZU_MC_TABLES_H", "azu_tables"))
    print("ok: 256 rows, edge masks match the crossing rule")


if __name__ == "__main__":
    main()
