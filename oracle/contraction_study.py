"""How often floating-point contraction changes the mesh: the CPU oracle built
as usual (every float operation rounded on its own, the arithmetic of the
CUDA path) against the same source built with multiply-adds contracted into
fused operations (-ffp-contract=fast).  The reference's CUDA is compiled with
nvcc's default contraction, whose choices cannot be read off; this measures
how sensitive the topology is to such a change at all, on seeded grids of the
workloads' kinds.  Test infrastructure (the oracle only; no GPU).

Usage: python oracle/contraction_study.py [--quick]
"""
import argparse
import ctypes
import platform
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import _support as S  # noqa: E402
from manifolddmc_gb300.workloads import gaussian_blobs  # noqa: E402

CONTRACTED = HERE / "_build" / "libmdmc_oracle_contracted.so"


def build_contracted():
    flags = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=fast", "-fno-fast-math"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # fused multiply-add instructions (aarch64 has them by default)
    CONTRACTED.parent.mkdir(exist_ok=True)
    subprocess.run(["g++", *flags, "-shared", "-o", str(CONTRACTED), str(HERE / "dmc_oracle.cpp")], check=True)
    return S._bind(ctypes.CDLL(str(CONTRACTED)))


def run(lib, vol, iso, refine=0, pad=False):
    dims = [vol.shape[2], vol.shape[1], vol.shape[0]]
    z3, o3 = np.zeros(3, np.float32), np.ones(3, np.float32)
    saved = S.oracle
    S.oracle = lambda: lib
    try:
        if refine or pad:
            return S.oracle_run_refined(vol.reshape(-1), dims, z3, o3, refine, pad, iso)
        return S.oracle_run(vol.reshape(-1), dims, z3, o3, iso)
    finally:
        S.oracle = saved


def compare(a, b):
    out = {"faces": (len(a["face_first"]), len(b["face_first"])),
           "vertices": (len(a["positions"]), len(b["positions"]))}
    same_dmc = (a["dmc_quads"].shape == b["dmc_quads"].shape and np.array_equal(a["dmc_quads"], b["dmc_quads"]))
    out["dmc_quads_identical"] = bool(same_dmc)
    if a["dmc_quads"].shape == b["dmc_quads"].shape:
        out["dmc_quads_differing"] = int(np.any(a["dmc_quads"] != b["dmc_quads"], axis=1).sum())
    if a["dmc_positions"].shape == b["dmc_positions"].shape:
        d = np.abs(a["dmc_positions"].astype(np.float64) - b["dmc_positions"].astype(np.float64))
        out["dmc_position_max_diff"] = float(np.nanmax(d)) if d.size else 0.0
    same_final = (a["halfedges"].shape == b["halfedges"].shape and np.array_equal(a["halfedges"], b["halfedges"]))
    out["final_halfedges_identical"] = bool(same_final)
    out["stats_identical"] = a["stats"] == b["stats"]
    for k in ("edges4", "nm_vertices", "split_iterations"):
        out[k] = (a["stats"][k], b["stats"][k])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="smaller grids only")
    args = ap.parse_args()
    strict = S.oracle()
    fused = build_contracted()
    rng = np.random.default_rng(7)
    cases = [
        ("blobs 65^3 refined x4 (257^3 samples)", gaussian_blobs(65, 16, (2.0, 8.0), seed=3), 0.4, 3, False),
        ("blobs 129^3", gaussian_blobs(129, 64, (3.0, 12.0), seed=1), 0.4, 0, False),
        ("noise 64^3", rng.random((64, 64, 64), dtype=np.float32), 0.5, 0, False),
        ("noise 96^3", rng.random((96, 96, 96), dtype=np.float32), 0.5, 0, False),
    ]
    if not args.quick:
        cases.append(("noise 128^3", rng.random((128, 128, 128), dtype=np.float32), 0.5, 0, False))
    for name, vol, iso, refine, pad in cases:
        t0 = time.time()
        a = run(strict, vol, iso, refine, pad)
        b = run(fused, vol, iso, refine, pad)
        print("%-40s %s (%.0f s)" % (name, compare(a, b), time.time() - t0), flush=True)


if __name__ == "__main__":
    main()
