"""Standard Marching Cubes (mdmc_run_standard_mc; the older CLI version's
standard_mc, OriginalDMC/src/DualMarchingCubes.cu:201-328) against the
oracle's restatement on the same refined grid: vertex positions, normals and
triangles bit-exact, in the same (edge-id, cell) order.  Structural checks on a
closed surface: every edge of the triangle mesh has exactly two triangles and
every normal has unit length."""
import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from _support import golden_grid, oracle_refine, oracle_standard_mc, reference_goldens, sphere_sdf
from test_gpu_parity import same_floats

pytestmark = pytest.mark.gpu


def _blobs(n, count, seed):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    v = np.zeros((n, n, n), np.float64)
    for _ in range(count):
        c = rng.uniform(0, n - 1, 3)
        s = rng.uniform(2.0, 5.0)
        v += np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    return v.astype(np.float32)


CASES = [
    # name, volume factory, iso, refinement, pad
    ("noise16", lambda: np.random.default_rng(31).random((16, 16, 16), dtype=np.float32), 0.5, 0, False),
    ("blobs24_pad", lambda: _blobs(24, 6, 32), 0.4, 0, True),
    ("blobs13_refine3", lambda: _blobs(13, 4, 33), 0.4, 3, False),
    ("noise9x14x11_refine1_pad", lambda: np.random.default_rng(34).random((11, 14, 9), dtype=np.float32), 0.45, 1, True),
]


def _compare(vol, dims, origin, spacing, iso, refinement, pad, nonempty=True):
    grid = mdmc.UniformGrid(np.ascontiguousarray(vol, np.float32).reshape(dims[2], dims[1], dims[0]), dims, origin,
                            spacing, refinement, pad)
    dmc = mdmc.DualMarchingCubes()
    pos, nrm, tri = dmc.run_standard_mc(iso, grid)
    g, d, o, s = oracle_refine(vol.reshape(-1), dims, origin, spacing, refinement, pad)
    rpos, rnrm, rtri = oracle_standard_mc(g, d, o, s, iso)
    assert pos.shape == rpos.shape and tri.shape == rtri.shape
    assert len(tri) > 0 or not nonempty
    assert same_floats(pos, rpos)
    assert same_floats(nrm, rnrm)
    assert np.array_equal(tri, rtri)
    return dmc, pos, nrm, tri


@pytest.mark.parametrize("name,factory,iso,refinement,pad", CASES, ids=[c[0] for c in CASES])
def test_standard_mc_matches_oracle(name, factory, iso, refinement, pad):
    vol = factory()
    dims = [vol.shape[2], vol.shape[1], vol.shape[0]]
    _compare(vol, dims, np.array([0.5, -1.0, 2.0], np.float32), np.array([0.25, 0.5, 1.0], np.float32), iso,
             refinement, pad)


@pytest.mark.parametrize("case", sorted(reference_goldens().keys()))
def test_standard_mc_reference_grids(case):
    samples, dims, origin, spacing, iso = golden_grid(case)
    _compare(samples, dims, origin, spacing, iso, 0, True)


def test_standard_mc_keeps_the_dmc_mesh_and_closes_a_sphere():
    n = 48
    vol = sphere_sdf(n, 0.35 * n)
    dims = [n, n, n]
    grid = mdmc.UniformGrid(vol, dims)
    dmc = mdmc.DualMarchingCubes()
    dmc.run(0.0, grid)
    before = dmc.get_halfedge_mesh()
    pos, nrm, tri = dmc.run_standard_mc(0.0, grid)
    after = dmc.get_halfedge_mesh()
    assert np.array_equal(before.halfedges, after.halfedges)
    assert np.array_equal(before.positions.view(np.uint32), after.positions.view(np.uint32))
    # closed 2-manifold: every undirected edge in exactly two triangles,
    # each directed edge once (consistent orientation)
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
    und = np.sort(e, axis=1)
    _, counts = np.unique(und, axis=0, return_counts=True)
    assert np.all(counts == 2)
    assert len(np.unique(e, axis=0)) == len(e)
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-5)
    # Euler characteristic of a sphere
    assert len(pos) - len(und) // 2 + len(tri) == 2


def test_standard_mc_without_crossing_is_empty():
    vol = np.ones((6, 7, 8), np.float32)
    grid = mdmc.UniformGrid(vol, [8, 7, 6])
    dmc = mdmc.DualMarchingCubes()
    pos, nrm, tri = dmc.run_standard_mc(0.5, grid)
    assert pos.shape == (0, 3) and tri.shape == (0, 3)


def _sweep_cases(n=40, seed=77):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = [int(rng.integers(2, 24)) for _ in range(3)]
        kind = ["noise", "quantised", "blobs"][i % 3]
        out.append(("%02d_%s_%dx%dx%d" % (i, kind, *dims), kind, dims, int(rng.integers(0, 2**31)),
                    int(rng.choice([0, 0, 1, 3])), bool(rng.integers(0, 2))))
    return out


SWEEP = _sweep_cases()


@pytest.mark.parametrize("name,kind,dims,seed,refinement,pad", SWEEP, ids=[c[0] for c in SWEEP])
def test_standard_mc_sweep(name, kind, dims, seed, refinement, pad):
    rng = np.random.default_rng(seed)
    shape = (dims[2], dims[1], dims[0])
    if kind == "noise":
        vol = rng.random(shape, dtype=np.float32)
    elif kind == "quantised":
        vol = (rng.integers(0, 5, shape) * 0.25).astype(np.float32)
    else:
        vol = _blobs(max(dims), 3, seed % 1000)[:dims[2], :dims[1], :dims[0]].copy()
    _compare(vol, dims, np.array([-0.5, 1.0, 0.25], np.float32), np.array([0.75, 0.5, 1.25], np.float32),
             0.5 if kind != "blobs" else 0.3, refinement, pad, nonempty=False)
