"""mdmc_run_to_host: the run with its mesh copied to caller-owned host
arrays while the later stages run.  The host arrays must equal what
mdmc_run + mdmc_download_mesh give, bit for bit, whether the copies made
after the quad and vertex passes stay valid (no repair) or a repair stage
rewrites the mesh afterwards (twin reconnection, splitter, simplification)."""
import numpy as np
import pytest

import manifolddmc_gb300 as mdmc

pytestmark = pytest.mark.gpu

FIELDS = ["positions", "normals", "quads", "halfedges", "face_first_halfedge", "face_attributes", "vertex_halfedge",
          "vertex_flags"]


def _blobs(n, count, seed):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    v = np.zeros((n, n, n), np.float64)
    for _ in range(count):
        c = rng.uniform(0, n - 1, 3)
        s = rng.uniform(2.0, 5.0)
        v += np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    return v.astype(np.float32)


def _noise(n, seed):
    return np.random.default_rng(seed).random((n, n, n), dtype=np.float32)


CASES = [
    # name, volume, iso, refinement, pad, flags
    ("blobs33_refine3", lambda: _blobs(33, 8, 51), 0.4, 3, False, {}),
    ("noise24_split", lambda: _noise(24, 52), 0.5, 0, False, {}),
    ("noise24_no_split", lambda: _noise(24, 53), 0.5, 0, False, {"split_non_manifold_halfedges": 0}),
    ("noise20_simplify", lambda: _noise(20, 54), 0.5, 0, True, {"simplify_p3x3y_color": 1, "simplify_p3333": 1}),
]


def _equal(a, b):
    for f in FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        assert x.shape == y.shape, f
        assert np.array_equal(np.ascontiguousarray(x).view(np.uint8), np.ascontiguousarray(y).view(np.uint8)), f


@pytest.mark.parametrize("name,factory,iso,refinement,pad,flags", CASES, ids=[c[0] for c in CASES])
def test_run_to_host_matches_run_and_download(name, factory, iso, refinement, pad, flags):
    vol = factory()
    dims = [vol.shape[2], vol.shape[1], vol.shape[0]]
    grid = mdmc.UniformGrid(vol, dims, (0.5, -1.0, 2.0), (0.25, 0.5, 1.0), refinement, pad)
    ref = mdmc.DualMarchingCubes(**flags)
    ref.run(iso, grid)
    expect = ref.get_halfedge_mesh()
    dmc = mdmc.DualMarchingCubes(**flags)
    host = mdmc.HostMesh(len(expect.positions) + 7, len(expect.quads) + 5)
    for _ in range(2):  # twice into the same host arrays
        got = dmc.run_to_host(iso, grid, host)
        _equal(got, expect)
        assert dmc.stats.num_edges4 == ref.stats.num_edges4
        assert dmc.stats.split_iterations == ref.stats.split_iterations


def test_run_to_host_rejects_small_host_arrays_and_keeps_the_device_mesh():
    vol = _noise(16, 55)
    grid = mdmc.UniformGrid(vol, [16, 16, 16])
    dmc = mdmc.DualMarchingCubes()
    host = mdmc.HostMesh(10, 10)
    with pytest.raises(mdmc.MDMCError) as e:
        dmc.run_to_host(0.5, grid, host)
    assert e.value.status == 4 and "host arrays hold 10 and 10" in str(e.value)
    ref = mdmc.DualMarchingCubes()
    ref.run(0.5, grid)
    _equal(dmc.get_halfedge_mesh(), ref.get_halfedge_mesh())


def test_run_to_host_with_pageable_arrays_and_null_fields():
    """Plain (pageable) numpy arrays work too, and a NULL array is skipped."""
    import ctypes
    vol = _blobs(20, 4, 56)
    grid = mdmc.UniformGrid(vol, [20, 20, 20], refinement=1)
    ref = mdmc.DualMarchingCubes()
    ref.run(0.4, grid)
    expect = ref.get_halfedge_mesh()
    V, F = len(expect.positions), len(expect.quads)
    arrays = {"positions": np.zeros((V, 3), np.float32), "normals": None, "quads": np.zeros((F, 4), np.int32),
              "halfedges": np.zeros((4 * F, 4), np.int32), "face_first_halfedge": np.zeros(F, np.int32),
              "face_attributes": None, "vertex_halfedge": np.zeros(V, np.int32), "vertex_flags": np.zeros(V, np.uint8)}
    host = mdmc.HostMeshArrays(V, F, *[a.ctypes.data if a is not None else None for a in arrays.values()])
    dmc = mdmc.DualMarchingCubes()
    st = dmc._ctx.lib.mdmc_run_to_host(dmc._ctx.handle, ctypes.byref(grid.grid), ctypes.c_float(0.4),
                                       ctypes.byref(host), ctypes.byref(dmc.mesh), ctypes.byref(dmc.stats), None)
    assert st == 0
    for k, a in arrays.items():
        if a is not None:
            assert np.array_equal(a, getattr(expect, k)), k
