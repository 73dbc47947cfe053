"""Recipe: re-encode the reference's Marching Cubes polygon table.

The Dual Marching Cubes path of the reference reads its cell polygons from
``s_polygonPatterns`` (MarchingCubes/VisualDMC/src/DMC/DualMarchingCubes.cpp:564)
and its ambiguity marks from ``s_triangleAmbiguities`` (same file, :301).
The per-cell vertex positions are sums of edge crossings taken in the table's
edge order, so bit-exact parity needs the same contour and edge order.  This
script stores that order in the packed 64-bit layout that the reference builds
at run time in ``Contour`` (D/CellIntersection.h:28-137): contour sizes in
nibbles 0-3, the edges of all contours back to back in nibbles 4-15.  One
8-byte word per case replaces a 17-byte row walk in the cell kernel.

It writes the same words to the product header and to the oracle's header,
and a SHA-256 digest of the words and of the ambiguity marks to
``tests/golden/mc_tables_digest.json`` so that the tests can check both
headers (and the ambiguity rule written in code) without the reference.

The standard Marching Cubes path reads the triangle table of the older CLI
version (``t_pattern``, MarchingCubes/OriginalDMC/src/DualMarchingCubes.h:160)
with its intersected-edge masks (``e_pattern``, :123).  Each case's triangles
are packed into one 64-bit word: bits 0-3 the triangle count, then the cell
edges of the triangles, three per triangle, one nibble each, in table order.

Run from the repository root:  python3 oracle/gen_mc_tables.py <reference_root>
(or with the reference checkout named by the environment variable MDMC_REFERENCE).
"""
import hashlib
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MDMC_REFERENCE")
if not REF:
    sys.exit("usage: %s <reference_root>  (or set MDMC_REFERENCE)" % sys.argv[0])
SRC = os.path.join(REF, "MarchingCubes/VisualDMC/src/DMC/DualMarchingCubes.cpp")
SRC_MC = os.path.join(REF, "MarchingCubes/OriginalDMC/src/DualMarchingCubes.h")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _array(src, name):
    i = src.index(name)
    j = src.index("{", i)
    k = src.index("};", j)
    body = re.sub(r"//[^\n]*", "", src[j + 1:k])
    body = body.replace("MC_AMBIGUOUS", "105")
    body = re.sub(r"static_cast<char>\((-?\d+)\)", r"\1", body)
    return [int(t) for t in re.findall(r"-?\d+", body)]


def pack_case(row):
    n = row[0]
    word = 0xFFFFFFFFFFFF0000
    cursor = n + 1
    total = 0
    for t in range(n):
        size = row[1 + t]
        word &= ~(0xF << (4 * t))
        word |= size << (4 * t)
        for i in range(size):
            bit = 16 + 4 * (total + i)
            word &= ~(0xF << bit)
            word |= row[cursor] << bit
            cursor += 1
        total += size
    return word & 0xFFFFFFFFFFFFFFFF


def main():
    src = open(SRC, encoding="latin-1").read()
    poly = _array(src, "s_polygonPatterns =")
    amb = _array(src, "s_triangleAmbiguities =")
    assert len(poly) == 256 * 17 and len(amb) == 256
    words = [pack_case(poly[17 * c:17 * c + 17]) for c in range(256)]
    ambiguous = [1 if amb[c] == 105 else 0 for c in range(256)]

    lines = []
    for c in range(0, 256, 4):
        lines.append("    " + ", ".join("0x%016xULL" % w for w in words[c:c + 4]) + ",")
    table = "\n".join(lines)
    header = (
        "// Generated by oracle/gen_mc_tables.py -- do not edit by hand.\n"
        "// Per Marching Cubes case (bit i set <=> corner i >= iso), the cell's\n"
        "// contours packed as: nibbles 0-3 = contour sizes, nibbles 4-15 = the\n"
        "// intersected cell edges of all contours back to back (0xF = unused).\n"
        "// Same contour/edge order as the reference's polygon table\n"
        "// (MarchingCubes/VisualDMC/src/DMC/DualMarchingCubes.cpp:564), packed as\n"
        "// its Contour class does (D/CellIntersection.h:28-137).  Ambiguous cases\n"
        "// do not read this table.\n"
    )
    prod = os.path.join(ROOT, "manifolddmc_gb300", "csrc", "mc_contour_table.h")
    with open(prod, "w") as f:
        f.write("#pragma once\n" + header +
                "#define MDMC_CONTOUR_WORDS \\\n" + table.replace(",\n", ", \\\n").rstrip(",") + "\n\n"
                "namespace mdmc {\n// Lives in global memory; kernels stage it in shared memory (lanes index it\n"
                "// with divergent cases, which would serialise a __constant__ read).\n"
                "__device__ const unsigned long long kContourTable[256] = {MDMC_CONTOUR_WORDS};\n"
                "static const unsigned long long kContourTableHost[256] = {MDMC_CONTOUR_WORDS};\n"
                "}  // namespace mdmc\n")
    orc = os.path.join(ROOT, "oracle", "mc_contour_table_oracle.h")
    with open(orc, "w") as f:
        f.write("#pragma once\n" + header +
                "namespace oracle {\nstatic const unsigned long long kContourTable[256] = {\n"
                + table + "\n};\n}  // namespace oracle\n")
    digest = {
        "contour_words_sha256": hashlib.sha256(
            b"".join(w.to_bytes(8, "little") for w in words)).hexdigest(),
        "ambiguous_sha256": hashlib.sha256(bytes(ambiguous)).hexdigest(),
        "num_ambiguous": sum(ambiguous),
        "source": "MarchingCubes/VisualDMC/src/DMC/DualMarchingCubes.cpp:301,564",
    }
    # standard Marching Cubes triangle table (OriginalDMC)
    src_mc = open(SRC_MC, encoding="latin-1").read()
    e_pat = _array(src_mc, "e_pattern = std::array")
    t_pat = _array(src_mc, "t_pattern = std::array")
    assert len(e_pat) == 256 and len(t_pat) == 4096
    tri_words = []
    for c in range(256):
        row = t_pat[16 * c:16 * c + 16]
        n = 0
        while n < 5 and row[3 * n] != -1:
            n += 1
        w = n
        for k in range(3 * n):
            assert 0 <= row[k] < 12
            w |= row[k] << (4 + 4 * k)
        tri_words.append(w)
    tlines = []
    for c in range(0, 256, 4):
        tlines.append("    " + ", ".join("0x%016xULL" % w for w in tri_words[c:c + 4]) + ",")
    ttable = "\n".join(tlines)
    theader = (
        "// Generated by oracle/gen_mc_tables.py -- do not edit by hand.\n"
        "// Standard Marching Cubes triangles per case (bit i set <=> corner i >= iso):\n"
        "// bits 0-3 = number of triangles, then 3 cell edges per triangle, one nibble\n"
        "// each, in the order of the reference's t_pattern\n"
        "// (MarchingCubes/OriginalDMC/src/DualMarchingCubes.h:160).\n"
    )
    with open(os.path.join(ROOT, "manifolddmc_gb300", "csrc", "mc_triangle_table.h"), "w") as f:
        f.write("#pragma once\n" + theader + "namespace mdmc {\n"
                "__device__ const unsigned long long kTriangleTable[256] = {\n" + ttable + "\n};\n"
                "static const unsigned long long kTriangleTableHost[256] = {\n" + ttable + "\n};\n"
                "}  // namespace mdmc\n")
    with open(os.path.join(ROOT, "oracle", "mc_triangle_table_oracle.h"), "w") as f:
        f.write("#pragma once\n" + theader + "namespace oracle {\nstatic const unsigned long long kTriangleTable[256] = {\n"
                + ttable + "\n};\n}  // namespace oracle\n")
    digest["triangle_words_sha256"] = hashlib.sha256(b"".join(w.to_bytes(8, "little") for w in tri_words)).hexdigest()
    digest["edge_patterns_sha256"] = hashlib.sha256(b"".join(v.to_bytes(2, "little") for v in e_pat)).hexdigest()
    digest["triangle_source"] = "MarchingCubes/OriginalDMC/src/DualMarchingCubes.h:123,160"
    with open(os.path.join(ROOT, "tests", "golden", "mc_tables_digest.json"), "w") as f:
        json.dump(digest, f, indent=1)
        f.write("\n")
    print("wrote", prod, orc, digest)


if __name__ == "__main__":
    main()
