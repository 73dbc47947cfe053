"""Writes tests/golden/noise256_digest.json: SHA-256 digests of every output
array and the statistics of the CPU oracle on the 256^3 uniform-noise
workload (manifolddmc_gb300.workloads.CONFIGS["noise256"]: iid uniform[0, 1]
noise, seed 1, iso 0.5, origin 0, spacing 1, the reference's default flags).

The oracle's halfedge build and repair are sequential, so a run takes several
minutes; the GPU test compares the library's arrays against these digests at
the full size instead of running the oracle again.

Usage: python tests/golden/make_noise_digests.py
"""
import hashlib
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from _support import face_vertices, oracle_run  # noqa: E402
from manifolddmc_gb300.workloads import CONFIGS  # noqa: E402

CANONICAL_NAN = np.uint32(0x7FC00000)


def array_digest(a):
    """SHA-256 of an array's bytes (C order); float32 arrays with every NaN
    written as 0x7FC00000 (a normal of a zero gradient is 0/0, whose bit
    pattern differs between the GPU and the host)."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        bits = a.view(np.uint32).copy()
        bits[np.isnan(a)] = CANONICAL_NAN
        a = bits
    return {"sha256": hashlib.sha256(a.tobytes()).hexdigest(), "shape": list(a.shape), "dtype": str(a.dtype)}


def main():
    name = "noise256"
    desc, gen, iso, refine, pad = CONFIGS[name]
    assert refine == 0 and not pad
    vol = gen()
    dims = [vol.shape[2], vol.shape[1], vol.shape[0]]
    t0 = time.time()
    ref = oracle_run(vol.reshape(-1), dims, np.zeros(3, np.float32), np.ones(3, np.float32), iso)
    secs = time.time() - t0
    quads = face_vertices(ref["halfedges"], ref["face_first"]).astype(np.int32)
    out = {
        "workload": name,
        "description": desc,
        "dims": dims,
        "iso": iso,
        "oracle_seconds": round(secs, 1),
        "counts": {"vertices": len(ref["positions"]), "faces": len(ref["face_first"]),
                   "halfedges": len(ref["halfedges"]), "dmc_vertices": len(ref["dmc_positions"]),
                   "dmc_quads": len(ref["dmc_quads"])},
        "stats": ref["stats"],
        "arrays": {
            "positions": array_digest(ref["positions"]),
            "normals": array_digest(ref["normals"]),
            "halfedges": array_digest(ref["halfedges"]),
            "face_first_halfedge": array_digest(ref["face_first"]),
            "face_attributes": array_digest(ref["face_attr"]),
            "vertex_flags": array_digest(ref["vertex_flags"]),
            "vertex_halfedge": array_digest(ref["vertex_he"]),
            "quads": array_digest(quads),
        },
    }
    path = HERE / ("%s_digest.json" % name)
    path.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote %s (oracle %.0f s)" % (path, secs))


if __name__ == "__main__":
    main()
