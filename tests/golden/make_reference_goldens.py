"""Recipe: turn the reference's golden problems and meshes into one fixture.

Reads Data-and-Results/Base-Problems/*.bin (uint16 volumes) and the four
result levels in Data-and-Results/Base-Results/ (OBJ meshes written by
Mesh::writeToFile, MarchingCubes/VisualDMC/src/DMC/Mesh.cu:446-510) of
PhiliGuertler/ManifoldDMC and writes tests/golden/reference_goldens.json:

  {case: {"dims", "spacing", "samples", "iso",
          "levels": {"0".."3": {"v": [[x,y,z]...], "vn": [...], "f": [[a,b,c,d]...]}}}}

Face indices are converted to 0-based.  Levels (Data-and-Results/README.md,
MarchingCubes/VisualDMC/src/LayerCUDA.cpp:575-636):
  0 = no padding, no split; 1 = padding, no split;
  2 = padding, one splitter iteration; 3 = padding, full splitter.

Run from the repository root:  python3 tests/golden/make_reference_goldens.py <reference_root>
(or with the reference checkout named by the environment variable MDMC_REFERENCE).
"""
import json
import os
import struct
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MDMC_REFERENCE")
if not REF:
    sys.exit("usage: %s <reference_root>  (or set MDMC_REFERENCE)" % sys.argv[0])
DR = os.path.join(REF, "Data-and-Results")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")

CASES = {
    # case name: (problem file, result file stem for levels 0-1, for levels 2-3, iso)
    "1-Edge": ("1-Edge.bin", "1-Edge", "1-Edge", 900.0),
    "2-Edge": ("2-Edge.bin", "2-Edge", "2-Edge", 900.0),
    "3-Edge": ("3-Edge.bin", "3-Edge", "3-Edge", 900.0),
    "4-Edge": ("4-Edge.bin", "4-Edge", "4-Edge", 900.0),
    "Iterative-Fix": ("Iterative-Fix.bin", "Iterative-Fix", "Iteration-Fix", 900.0),
    "Non-Manifold-Vertex": ("Non-Manifold-Vertex.bin", "Non-Manifold-Vertex", "Non-Manifold-Vertex", 900.0),
    "12-Merge": ("12-Merge-iso-241.525.bin", "12-Merge", "12-Merge", 241.525),
}
LEVEL_DIRS = ["0_No-Fixes", "1_Grid-Extension-Fix", "2_One-Iteration", "3_Fully-Fixed"]


def read_obj(path):
    v, vn, f = [], [], []
    for line in open(path):
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            v.append([float(x) for x in t[1:4]])
        elif t[0] == "vn":
            vn.append([float(x) for x in t[1:4]])
        elif t[0] == "f":
            f.append([int(x.split("/")[0]) - 1 for x in t[1:5]])
    return {"v": v, "vn": vn, "f": f}


def main():
    out = {}
    for name, (binf, stem01, stem23, iso) in CASES.items():
        raw = open(os.path.join(DR, "Base-Problems", binf), "rb").read()
        dims = list(struct.unpack("3i", raw[:12]))
        spacing = list(struct.unpack("3f", raw[12:24]))
        n = dims[0] * dims[1] * dims[2]
        samples = list(struct.unpack("%dH" % n, raw[24:24 + 2 * n]))
        levels = {}
        for lvl, d in enumerate(LEVEL_DIRS):
            stem = stem01 if lvl < 2 else stem23
            levels[str(lvl)] = read_obj(os.path.join(DR, "Base-Results", d, stem + ".obj"))
        out[name] = {"dims": dims, "spacing": spacing, "samples": samples, "iso": iso,
                     "source": "Data-and-Results/Base-Problems/" + binf, "levels": levels}
    with open(OUT, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
