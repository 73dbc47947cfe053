"""Shared helpers for the test-suite: the CPU oracle's ctypes binding, golden
fixtures and mesh canonicalisation.  The oracle is test infrastructure; the
product library (manifolddmc_gb300) never loads it."""
import ctypes
import json
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
ORACLE_SO = ORACLE_DIR / "_build" / "libmdmc_oracle.so"
ORACLE_F64_SO = ORACLE_DIR / "_build" / "libmdmc_oracle_f64.so"
GOLDEN_DIR = ROOT / "tests" / "golden"

_lock = threading.Lock()
_lib = None
_lib64 = None

# SplittingStep, MarchingCubes/VisualDMC/src/DMC/PostProcesses/ManifoldSplitter.h:155-166
STEP_NONE, STEP_SUBDIVIDE, STEP_COLLAPSE, STEP_MERGE, STEP_TWINS, STEP_MOVE, STEP_ITERATE = range(7)
STEP_ALL = 100

STAT_NAMES = ["edges", "edges3", "edges4", "nm_vertices", "quads_nm1", "quads_nm2",
              "quads_nm3", "quads_nm4", "split_iterations", "anomalies"]


class OracleOptions(ctypes.Structure):
    _fields_ = [("surface_iteration", ctypes.c_int),
                ("simplify_3x3y_color", ctypes.c_int),
                ("simplify_3x3y_old", ctypes.c_int),
                ("simplify_3333", ctypes.c_int),
                ("split_non_manifold", ctypes.c_int),
                ("detect_non_manifold_vertices", ctypes.c_int),
                ("splitting_step", ctypes.c_int)]


def build_oracle():
    """Builds oracle/_build/libmdmc_oracle.so (and its FP64 build
    libmdmc_oracle_f64.so) when missing or stale."""
    srcs = [ORACLE_DIR / n for n in ("dmc_oracle.cpp", "dmc_oracle.h", "mc_contour_table_oracle.h",
                                     "mc_triangle_table_oracle.h", "Makefile")]
    if all(so.exists() and all(so.stat().st_mtime >= s.stat().st_mtime for s in srcs)
           for so in (ORACLE_SO, ORACLE_F64_SO)):
        return
    subprocess.run(["make", "-s", "-j2", "-C", str(ORACLE_DIR)], check=True)


def oracle():
    """The float restatement (bit for bit the CUDA path's arithmetic)."""
    global _lib
    with _lock:
        if _lib is None:
            build_oracle()
            _lib = _bind(ctypes.CDLL(str(ORACLE_SO)))
    return _lib


def oracle_f64():
    """The same restatement computing in double (the timed FP64 CPU baseline)."""
    global _lib64
    with _lock:
        if _lib64 is None:
            build_oracle()
            _lib64 = _bind(ctypes.CDLL(str(ORACLE_F64_SO)))
    return _lib64


def _bind(lib):
    """Declares the argument and result types of the oracle library's C API."""
    lib.mdmc_oracle_run.restype = ctypes.c_void_p
    lib.mdmc_oracle_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p]
    for name in ("mdmc_oracle_counts", "mdmc_oracle_stats", "mdmc_oracle_free"):
        getattr(lib, name).argtypes = [ctypes.c_void_p] + ([ctypes.c_void_p] if name != "mdmc_oracle_free" else [])
    lib.mdmc_oracle_get.argtypes = [ctypes.c_void_p] * 8
    lib.mdmc_oracle_get_dmc.argtypes = [ctypes.c_void_p] * 5
    lib.mdmc_oracle_refine.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]
    lib.mdmc_oracle_read_bin.argtypes = [ctypes.c_char_p] + [ctypes.c_void_p] * 4
    lib.mdmc_oracle_get_topology.argtypes = [ctypes.c_void_p] * 4
    lib.mdmc_oracle_standard_mc.restype = ctypes.c_void_p
    lib.mdmc_oracle_standard_mc.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_float, ctypes.c_void_p]
    lib.mdmc_oracle_get_standard_mc.argtypes = [ctypes.c_void_p] * 4
    lib.mdmc_oracle_free_standard_mc.argtypes = [ctypes.c_void_p]
    lib.mdmc_oracle_color_faces.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int64]
    lib.mdmc_oracle_quads_to_triangles.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    lib.mdmc_oracle_mean_ratio.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    lib.mdmc_oracle_positions_f64.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_double, ctypes.c_void_p]
    lib.mdmc_oracle_backward.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_double, ctypes.c_void_p,
                                                                 ctypes.c_void_p]
    lib.mdmc_oracle_refine_f64.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p]
    lib.mdmc_oracle_refine_backward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_void_p]
    lib.mdmc_oracle_run_refined.restype = ctypes.c_void_p
    lib.mdmc_oracle_run_refined.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                                    ctypes.c_void_p]
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def default_options(**kw):
    o = OracleOptions(1, 0, 0, 0, 1, 1, STEP_ALL)
    for k, v in kw.items():
        setattr(o, k, int(v))
    return o


def refined_geometry(dims, spacing, origin, refinement, pad):
    dims = np.asarray(dims, np.int64)
    out = dims + (dims - 1) * refinement + (2 if pad else 0)
    sp = (np.asarray(spacing, np.float32) * np.float32(1.0)) / (np.float32(refinement) + np.float32(1.0))
    org = np.asarray(origin, np.float32).copy()
    if pad:
        org = (org - sp).astype(np.float32)
    return [int(x) for x in out], sp.astype(np.float32), org.astype(np.float32)


def oracle_refine(samples, dims, origin, spacing, refinement, pad):
    """samples: float32 array with x fastest; returns (grid, dims, origin, spacing)."""
    lib = oracle()
    samples = np.ascontiguousarray(samples, np.float32).reshape(-1)
    d = np.asarray(dims, np.int32)
    od, _, _ = refined_geometry(dims, spacing, origin, refinement, pad)
    out = np.empty(int(np.prod(od)), np.float32)
    odims = np.zeros(3, np.int32)
    oorg = np.zeros(3, np.float32)
    osp = np.zeros(3, np.float32)
    lib.mdmc_oracle_refine(_p(samples), _p(d), _p(np.asarray(origin, np.float32)),
                           _p(np.asarray(spacing, np.float32)), int(refinement), int(pad),
                           _p(out), _p(odims), _p(oorg), _p(osp))
    return out, [int(x) for x in odims], oorg, osp


def oracle_run(grid, dims, origin, spacing, iso, **opts):
    """Runs the oracle; returns a dict with the DMC stage and the final mesh."""
    lib = oracle()
    grid = np.ascontiguousarray(grid, np.float32).reshape(-1)
    assert grid.size == int(np.prod(dims))
    o = default_options(**opts)
    res = lib.mdmc_oracle_run(_p(grid), _p(np.asarray(dims, np.int32)),
                              _p(np.asarray(origin, np.float32)), _p(np.asarray(spacing, np.float32)),
                              ctypes.c_float(iso), ctypes.byref(o))
    return _collect(lib, res)


def oracle_run_refined(coarse, dims, origin, spacing, refinement, pad, iso, f64=False, **opts):
    """Refinement and run in one oracle call (the refined grid stays in the
    oracle's arithmetic type: float, or double with f64)."""
    lib = oracle_f64() if f64 else oracle()
    coarse = np.ascontiguousarray(coarse, np.float32).reshape(-1)
    assert coarse.size == int(np.prod(dims))
    o = default_options(**opts)
    res = lib.mdmc_oracle_run_refined(_p(coarse), _p(np.asarray(dims, np.int32)), _p(np.asarray(origin, np.float32)),
                                      _p(np.asarray(spacing, np.float32)), int(refinement), int(pad),
                                      ctypes.c_float(iso), ctypes.byref(o))
    return _collect(lib, res)


def _collect(lib, res):
    try:
        counts = np.zeros(5, np.int64)
        stats = np.zeros(10, np.int64)
        lib.mdmc_oracle_counts(res, _p(counts))
        lib.mdmc_oracle_stats(res, _p(stats))
        V, F, H, DV, DQ = (int(x) for x in counts)
        out = {
            "positions": np.zeros((V, 3), np.float32), "normals": np.zeros((V, 3), np.float32),
            "halfedges": np.zeros((H, 4), np.int32), "face_first": np.zeros(F, np.int32),
            "face_attr": np.zeros(F, np.uint16), "vertex_flags": np.zeros(V, np.uint8),
            "vertex_he": np.zeros(V, np.int32),
            "dmc_positions": np.zeros((DV, 3), np.float32), "dmc_normals": np.zeros((DV, 3), np.float32),
            "dmc_quads": np.zeros((DQ, 4), np.int32), "dmc_quad_attr": np.zeros(DQ, np.uint16),
        }
        lib.mdmc_oracle_get(res, _p(out["positions"]), _p(out["normals"]), _p(out["halfedges"]),
                            _p(out["face_first"]), _p(out["face_attr"]), _p(out["vertex_flags"]),
                            _p(out["vertex_he"]))
        lib.mdmc_oracle_get_dmc(res, _p(out["dmc_positions"]), _p(out["dmc_normals"]),
                                _p(out["dmc_quads"]), _p(out["dmc_quad_attr"]))
        out["stats"] = dict(zip(STAT_NAMES, (int(x) for x in stats)))
        return out
    finally:
        lib.mdmc_oracle_free(res)


def face_vertices(halfedges, face_first):
    """(F, 4) vertex ids of each face, walking next pointers from its first halfedge."""
    he = np.asarray(halfedges)
    h = np.asarray(face_first).astype(np.int64)
    cols = []
    for _ in range(4):
        cols.append(he[h, 0])
        h = he[h, 2]
    return np.stack(cols, axis=1) if len(face_first) else np.zeros((0, 4), np.int32)


# ---------------------------------------------------------------------------
# golden fixtures
# ---------------------------------------------------------------------------
_goldens = None


def reference_goldens():
    global _goldens
    if _goldens is None:
        with open(GOLDEN_DIR / "reference_goldens.json") as f:
            _goldens = json.load(f)
    return _goldens


LEVEL_OPTIONS = {
    # level: (pad, options) -- Data-and-Results/README.md, LayerCUDA.cpp:575-636
    0: (False, dict(split_non_manifold=0, splitting_step=STEP_NONE)),
    1: (True, dict(split_non_manifold=0, splitting_step=STEP_NONE)),
    2: (True, dict(split_non_manifold=1, splitting_step=STEP_MOVE)),
    3: (True, dict(split_non_manifold=1, splitting_step=STEP_ALL)),
}


def golden_grid(case):
    g = reference_goldens()[case]
    dims = g["dims"]
    spacing = np.asarray(g["spacing"], np.float32)
    origin = ((np.float32(-0.5) * (np.asarray(dims, np.float32) - np.float32(1))) * spacing).astype(np.float32)
    samples = np.asarray(g["samples"], np.float32)
    return samples, dims, origin, spacing, float(np.float32(g["iso"]))


def canonical_faces(faces):
    """Rotates each face to start at its smallest id (orientation kept) and sorts."""
    out = []
    for f in faces:
        f = list(int(x) for x in f)
        k = f.index(min(f))
        out.append(tuple(f[k:] + f[:k]))
    return sorted(out)


def match_to_golden(positions, faces, golden, tol):
    """Maps referenced vertices onto the golden mesh's vertices by position.
    Returns (mapped canonical faces, golden canonical faces, max distance, mapping)."""
    gv = np.asarray(golden["v"], np.float64)
    gf = np.asarray(golden["f"], np.int64).reshape(-1, 4)
    used = np.unique(np.asarray(faces).reshape(-1)) if len(faces) else np.zeros(0, np.int64)
    mapping = {}
    maxd = 0.0
    gref = np.unique(gf.reshape(-1)) if len(gf) else np.zeros(0, np.int64)
    for v in used:
        d = np.linalg.norm(gv[gref] - np.asarray(positions[v], np.float64)[None, :], axis=1)
        j = int(np.argmin(d))
        maxd = max(maxd, float(d[j]))
        mapping[int(v)] = int(gref[j])
    mapped = [[mapping[int(x)] for x in f] for f in faces]
    return canonical_faces(mapped), canonical_faces(gf), maxd, mapping


class OracleRun:
    """One oracle run kept open for the differentiable path: the DMC vertex
    topology (cell, contour edges), the parent DMC vertex of every final
    vertex, FP64 positions for a perturbed grid of the same dims and the FP64
    gradient of sum(dL/dpos . pos) with respect to the grid samples."""

    def __init__(self, grid, dims, origin, spacing, iso, **opts):
        self.lib = oracle()
        self.dims = np.asarray(dims, np.int32)
        self.origin = np.asarray(origin, np.float64)
        self.spacing = np.asarray(spacing, np.float64)
        self.iso = float(np.float32(iso))
        grid = np.ascontiguousarray(grid, np.float32).reshape(-1)
        o = default_options(**opts)
        self.res = self.lib.mdmc_oracle_run(_p(grid), _p(self.dims), _p(np.asarray(origin, np.float32)),
                                            _p(np.asarray(spacing, np.float32)), ctypes.c_float(iso),
                                            ctypes.byref(o))
        counts = np.zeros(5, np.int64)
        self.lib.mdmc_oracle_counts(self.res, _p(counts))
        self.num_vertices, self.num_dmc_vertices = int(counts[0]), int(counts[3])
        self.cells = np.zeros((self.num_dmc_vertices, 3), np.int32)
        self.edges = np.zeros(self.num_dmc_vertices, np.uint16)
        self.parents = np.zeros(self.num_vertices, np.int32)
        self.lib.mdmc_oracle_get_topology(self.res, _p(self.cells), _p(self.edges), _p(self.parents))
        self.positions = np.zeros((self.num_vertices, 3), np.float32)
        self.lib.mdmc_oracle_get(self.res, _p(self.positions), None, None, None, None, None, None)

    def positions_f64(self, grid64):
        out = np.zeros((self.num_dmc_vertices, 3), np.float64)
        g = np.ascontiguousarray(grid64, np.float64).reshape(-1)
        self.lib.mdmc_oracle_positions_f64(self.res, _p(g), _p(self.dims), _p(self.origin), _p(self.spacing),
                                           self.iso, _p(out))
        return out

    def backward(self, grid64, dLdpos):
        out = np.zeros(int(np.prod(self.dims)), np.float64)
        g = np.ascontiguousarray(grid64, np.float64).reshape(-1)
        d = np.ascontiguousarray(dLdpos, np.float64).reshape(-1)
        assert d.size == 3 * self.num_vertices
        self.lib.mdmc_oracle_backward(self.res, _p(g), _p(self.dims), _p(self.spacing), self.iso, _p(d), _p(out))
        return out

    def close(self):
        if self.res:
            self.lib.mdmc_oracle_free(self.res)
            self.res = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def refine_f64(coarse, dims, refinement, pad):
    od, _, _ = refined_geometry(dims, [1, 1, 1], [0, 0, 0], refinement, pad)
    out = np.zeros(int(np.prod(od)), np.float64)
    c = np.ascontiguousarray(coarse, np.float64).reshape(-1)
    oracle().mdmc_oracle_refine_f64(_p(c), _p(np.asarray(dims, np.int32)), int(refinement), int(pad), _p(out))
    return out


def refine_backward(dout, dims, refinement, pad):
    out = np.zeros(int(np.prod(dims)), np.float64)
    d = np.ascontiguousarray(dout, np.float64).reshape(-1)
    oracle().mdmc_oracle_refine_backward(_p(d), _p(np.asarray(dims, np.int32)), int(refinement), int(pad), _p(out))
    return out


def sphere_sdf(n, radius, center=None):
    """Signed distance to a sphere (cells), float32, x fastest."""
    c = (n - 1) / 2.0 if center is None else center
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return (np.sqrt((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2) - radius).astype(np.float32)


def oracle_standard_mc(grid, dims, origin, spacing, iso):
    """The oracle's standard Marching Cubes: (positions [V,3], normals [V,3], triangles [T,3])."""
    lib = oracle()
    grid = np.ascontiguousarray(grid, np.float32).reshape(-1)
    counts = np.zeros(2, np.int64)
    m = lib.mdmc_oracle_standard_mc(_p(grid), _p(np.asarray(dims, np.int32)), _p(np.asarray(origin, np.float32)),
                                    _p(np.asarray(spacing, np.float32)), ctypes.c_float(iso), _p(counts))
    try:
        V, T = int(counts[0]), int(counts[1])
        pos, nrm, tri = np.zeros((V, 3), np.float32), np.zeros((V, 3), np.float32), np.zeros((T, 3), np.int32)
        lib.mdmc_oracle_get_standard_mc(m, _p(pos), _p(nrm), _p(tri))
        return pos, nrm, tri
    finally:
        lib.mdmc_oracle_free_standard_mc(m)


def oracle_color_faces(halfedges, face_first, face_attr):
    """The oracle's 24 -> 5 face coloring; returns the new face attributes."""
    he = np.ascontiguousarray(halfedges, np.int32).reshape(-1, 4)
    ff = np.ascontiguousarray(face_first, np.int32)
    attr = np.array(face_attr, np.uint16, copy=True)
    oracle().mdmc_oracle_color_faces(_p(he), len(he), _p(ff), _p(attr), len(attr))
    return attr


def oracle_quads_to_triangles(quads):
    q = np.ascontiguousarray(quads, np.int32).reshape(-1, 4)
    t = np.zeros((2 * len(q), 3), np.int32)
    oracle().mdmc_oracle_quads_to_triangles(_p(q), len(q), _p(t))
    return t


def oracle_mean_ratio(positions, triangles):
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    tri = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    q = np.zeros(len(tri), np.float32)
    oracle().mdmc_oracle_mean_ratio(_p(pos), _p(tri), len(tri), _p(q))
    return q


# ---------------------------------------------------------------------------
# an independent manifold check (no oracle, no library code)
# ---------------------------------------------------------------------------
def manifold_report(halfedges, num_vertices, vertex_flags):
    """Recomputes, from the halfedge array alone, what the reference's
    statistics getters and fan detection report, with torch on whatever device
    the arrays are on (they are converted to torch tensors).

    - Edge valences: halfedges per undirected edge (min, max vertex), the
      edge table's count (D/Halfedges/HalfedgeMesh.cu:1164-1239).
    - Quads with k edges of valence > 2.
    - Face fans: the fans around a vertex are the connected components of its
      outgoing halfedges under h -> next(twin(h)) (one step of the cw walk of
      D/PostProcesses/ManifoldCreator.cu:393-465; the ccw step is its inverse
      where twins pair two opposite halfedges).  Found by pointer doubling
      forwards and backwards, so no walk is repeated.  Compared with the
      multi-fan flag only at "clean" vertices, whose incident edges all have 1
      or 2 halfedges (where a 3-halfedge edge's cyclic twins make the walk
      direction-dependent, the walk itself is the definition).

    Returns a dict of counts and the tensors the assertions use."""
    import torch

    he = torch.as_tensor(halfedges)
    dev = he.device
    H = he.shape[0]
    V = int(num_vertices)
    flags = torch.as_tensor(vertex_flags).to(dev)
    origin = he[:, 0].long()
    nxt = he[:, 2].long()
    twin = he[:, 3].long()
    dest = origin[nxt]
    lo = torch.minimum(origin, dest)
    hi = torch.maximum(origin, dest)
    key = lo * V + hi
    uniq, inv, counts = torch.unique(key, return_inverse=True, return_counts=True)
    valence = counts[inv]  # per halfedge
    # quads with k edges of valence > 2 (each halfedge names its face; after
    # the split a face's halfedges are no longer 4f..4f+3)
    face = he[:, 1].long()
    per_face = torch.bincount(face[valence > 2], minlength=int(face.max()) + 1 if H else 0)
    qk = [int((per_face == k).sum()) for k in range(1, 5)]
    # clean vertices: every incident edge has 1 or 2 halfedges
    bad = valence > 2
    unclean = torch.zeros(V, dtype=torch.bool, device=dev)
    unclean[origin[bad]] = True
    unclean[dest[bad]] = True
    # fan components: successor s(h) = next(twin(h)) when it leaves the same vertex
    idx = torch.arange(H, device=dev)
    has = twin >= 0
    cand = torch.where(has, nxt[torch.where(has, twin, 0)], idx)
    succ = torch.where(has & (origin[cand] == origin), cand, idx)
    pred = idx.clone()
    moved = succ != idx
    pred[succ[moved]] = idx[moved]

    def path_min(step):
        m = idx.clone()
        p = step.clone()
        for _ in range(40):  # 2^40 steps: any fan
            m2 = torch.minimum(m, m[p])
            p2 = p[p]
            if torch.equal(m2, m) and torch.equal(p2, p):
                break
            m, p = m2, p2
        return m

    fan_key = torch.minimum(path_min(succ), path_min(pred))
    is_key = fan_key == idx
    fans = torch.bincount(origin[is_key], minlength=V)
    multi = (flags & 8) != 0
    clean = ~unclean
    return {
        "num_edges": int(uniq.numel()),
        "edges_by_valence": {int(k): int(c) for k, c in zip(*torch.unique(counts, return_counts=True))},
        "quads_with_non_manifold_edges": qk,
        "num_flagged": int(multi.sum()),
        "clean_vertices": int(clean.sum()),
        "clean_mismatch": int(((fans > 1) != multi)[clean].sum()),
        "clean_multi_fan": int(((fans > 1) & clean).sum()),
        "twins_not_opposite_at_valence2": int(((valence == 2) & has & (origin[torch.where(has, twin, 0)] != dest)).sum()),
        "twins_not_involutive_at_valence2": int(((valence == 2) & has & (twin[torch.where(has, twin, 0)] != idx)).sum()),
    }
