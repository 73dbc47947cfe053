"""Builds the in-tree CUDA library manifolddmc_gb300/_build/libmdmc.so for sm_103a.

nvcc compiles the translation units in parallel and links one shared
library with the C ABI declared in include/mdmc.h.  -fmad=false keeps every
float operation separately rounded (the reference's expression order is kept
in the source), which the bit-exact parity with the CPU oracle relies on.
"""
import os
import shlex
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libmdmc.so"
SOURCES = ["mdmc_api.cu", "mdmc_dmc.cu", "mdmc_mesh.cu", "mdmc_split.cu", "mdmc_noalloc.cu", "mdmc_adjoint.cu", "mdmc_simplify.cu", "mdmc_batch.cu", "mdmc_generate.cu", "mdmc_mc.cu", "mdmc_quality.cu", "mdmc_points.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "-I", str(ROOT / "include"), "-I", str(CSRC)]


def nvcc():
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _stale():
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [ROOT / "include" / "mdmc.h"] + list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
    return any(d.stat().st_mtime > t for d in deps) or Path(__file__).stat().st_mtime > t


def build(force=False, verbose=False):
    """Compiles the library if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = OUT_DIR / (Path(src).stem + ".o")
        cmd = [cc] + ARCH + FLAGS + shlex.split(os.environ.get("MDMC_NVCC_FLAGS", "")) + ["-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = OUT_DIR / "libmdmc.so.tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
