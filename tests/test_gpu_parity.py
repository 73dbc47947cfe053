"""Parity of the CUDA path with the CPU oracle, through the C ABI.

Both sides follow the same deterministic ordering conventions and the same
float operation order (the library is built with -fmad=false, the oracle with
-ffp-contract=off), so every output array must be identical: positions and
normals bit for bit, halfedges, faces, attributes, flags and statistics
exactly.  The golden cases additionally tie both to the reference's meshes
(tests/test_oracle_golden.py pins the oracle to them).
"""
import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from _support import (LEVEL_OPTIONS, STEP_ALL, golden_grid, oracle_refine, oracle_run, reference_goldens)

pytestmark = pytest.mark.gpu

OPTION_MAP = {
    "surface_iteration": "enable_surface_to_vertex_iteration",
    "split_non_manifold": "split_non_manifold_halfedges",
    "detect_non_manifold_vertices": "detect_non_manifold_vertices",
    "splitting_step": "splitting_step",
    "simplify_3x3y_color": "simplify_p3x3y_color",
    "simplify_3x3y_old": "simplify_p3x3y_old",
    "simplify_3333": "simplify_p3333",
}


def gpu_run(samples, dims, origin, spacing, iso, refinement=0, pad=False, **opts):
    flags = {OPTION_MAP[k]: v for k, v in opts.items()}
    dmc = mdmc.DualMarchingCubes(**flags)
    grid = mdmc.UniformGrid(np.ascontiguousarray(samples, np.float32).reshape(dims[2], dims[1], dims[0]), dims,
                            origin, spacing, refinement, pad)
    dmc.run(iso, grid)
    m = dmc.get_halfedge_mesh()
    return dmc, m, grid


def oracle_for(samples, dims, origin, spacing, iso, refinement=0, pad=False, **opts):
    g, d, o, s = oracle_refine(samples, dims, origin, spacing, refinement, pad)
    return oracle_run(g, d, o, s, iso, **opts), (d, o, s)


def same_floats(a, b):
    """Bit-equal, except that any NaN equals any NaN: a normal of a zero
    gradient is 0/0, which the GPU writes as 0x7FFFFFFF and the host as
    0x7FC00000."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    if a.shape != b.shape:
        return False
    return bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))


def assert_parity(dmc, m, ref):
    assert m.positions.shape == ref["positions"].shape
    assert len(m.face_first_halfedge) == len(ref["face_first"])
    assert len(m.halfedges) == len(ref["halfedges"])
    assert same_floats(m.positions, ref["positions"])
    assert same_floats(m.normals, ref["normals"])
    assert np.array_equal(m.halfedges, ref["halfedges"])
    assert np.array_equal(m.face_first_halfedge, ref["face_first"])
    assert np.array_equal(m.face_attributes, ref["face_attr"])
    assert np.array_equal(m.vertex_flags, ref["vertex_flags"])
    assert np.array_equal(m.vertex_halfedge, ref["vertex_he"])
    st = ref["stats"]
    assert dmc.get_num_vertices() == len(ref["dmc_positions"])
    assert dmc.get_num_quads() == len(ref["dmc_quads"])
    assert dmc.get_num_edges() == st["edges"]
    assert dmc.get_num_non_manifold_edges3() == st["edges3"]
    assert dmc.get_num_non_manifold_edges4() == st["edges4"]
    assert dmc.get_num_non_manifold_vertices() == st["nm_vertices"]
    for k in range(1, 5):
        assert dmc.get_num_quads_with_non_manifold_edges(k) == st["quads_nm%d" % k]
    assert dmc.stats.split_iterations == st["split_iterations"]
    # identical device status word (limits hit, e.g. the fan-walk cap)
    assert dmc.stats.anomalies == st["anomalies"]
    # quads output = face walk
    if len(m.quads):
        he = m.halfedges
        h = m.face_first_halfedge.astype(np.int64)
        for i in range(4):
            assert np.array_equal(m.quads[:, i], he[h, 0])
            h = he[h, 2]


@pytest.mark.parametrize("level", [0, 1, 2, 3])
@pytest.mark.parametrize("case", list(reference_goldens().keys()))
def test_golden_cases_bit_exact(case, level):
    samples, dims, origin, spacing, iso = golden_grid(case)
    pad, opts = LEVEL_OPTIONS[level]
    dmc, m, _ = gpu_run(samples, dims, origin, spacing, iso, 0, pad, **opts)
    ref, _ = oracle_for(samples, dims, origin, spacing, iso, 0, pad, **opts)
    assert_parity(dmc, m, ref)


@pytest.mark.parametrize("case", list(reference_goldens().keys()))
def test_golden_grids_with_all_simplifications(case):
    # the reference's grids, padded, with every simplification before the repair
    samples, dims, origin, spacing, iso = golden_grid(case)
    opts = dict(simplify_3x3y_color=1, simplify_3x3y_old=1, simplify_3333=1)
    dmc, m, _ = gpu_run(samples, dims, origin, spacing, iso, 0, True, **opts)
    ref, _ = oracle_for(samples, dims, origin, spacing, iso, 0, True, **opts)
    assert_parity(dmc, m, ref)


def blobs(n, count, seed, sigma=(2.0, 5.0)):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    v = np.zeros((n, n, n), np.float64)
    for _ in range(count):
        c = rng.uniform(0, n - 1, 3)
        s = rng.uniform(*sigma)
        v += np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    return v.astype(np.float32)


RANDOM_CASES = [
    # name, volume factory, iso, refinement, pad, options
    ("noise16", lambda: np.random.default_rng(1).random((16, 16, 16), dtype=np.float32), 0.5, 0, False, {}),
    ("noise20_pad", lambda: np.random.default_rng(2).random((20, 20, 20), dtype=np.float32), 0.5, 0, True, {}),
    ("blobs24", lambda: blobs(24, 6, 3), 0.5, 0, True, {}),
    ("blobs17_refine3", lambda: blobs(17, 5, 4), 0.4, 3, False, {}),
    ("blobs13_refine1_pad", lambda: blobs(13, 4, 5), 0.45, 1, True, {}),
    ("noise14_nosurfiter", lambda: np.random.default_rng(6).random((14, 14, 14), dtype=np.float32), 0.5, 0, False,
     {"surface_iteration": 0}),
    ("noise14_nosplit", lambda: np.random.default_rng(7).random((14, 14, 14), dtype=np.float32), 0.5, 0, False,
     {"split_non_manifold": 0}),
    ("noise14_nodetect", lambda: np.random.default_rng(8).random((14, 14, 14), dtype=np.float32), 0.5, 0, False,
     {"detect_non_manifold_vertices": 0}),
    ("noise12x17x9", lambda: np.random.default_rng(9).random((9, 17, 12), dtype=np.float32), 0.5, 0, False, {}),
    # large refinement factors: coarse blocks of 13^3 (+ padding) refined cells
    # (evaluated two planes at a time), and beyond the block pass's plane size
    # (the row walk takes over)
    ("blobs7_refine12_pad", lambda: blobs(7, 3, 13, (1.0, 2.0)), 0.45, 12, True, {}),
    ("blobs7_refine19", lambda: blobs(7, 3, 12, (1.0, 2.5)), 0.4, 19, False, {}),
    # valence-pattern simplifications (HalfedgeMesh.cu:859-1048), alone and chained
    ("noise16_3x3y_color", lambda: np.random.default_rng(21).random((16, 16, 16), dtype=np.float32), 0.5, 0, False,
     {"simplify_3x3y_color": 1}),
    ("blobs32_3x3y_old_pad", lambda: blobs(32, 6, 3), 0.4, 0, True, {"simplify_3x3y_old": 1}),
    ("noise16_3333", lambda: np.random.default_rng(22).random((16, 16, 16), dtype=np.float32), 0.5, 0, False,
     {"simplify_3333": 1}),
    ("blobs28_all_simplify", lambda: blobs(28, 5, 23, (3.0, 7.0)), 0.3, 0, False,
     {"simplify_3x3y_color": 1, "simplify_3x3y_old": 1, "simplify_3333": 1}),
    ("blobs13_refine2_simplify", lambda: blobs(13, 4, 24), 0.4, 2, True,
     {"simplify_3x3y_color": 1, "simplify_3333": 1, "surface_iteration": 0}),
]


@pytest.mark.parametrize("name,factory,iso,refinement,pad,opts", RANDOM_CASES, ids=[c[0] for c in RANDOM_CASES])
def test_seeded_grids_bit_exact(name, factory, iso, refinement, pad, opts):
    vol = factory()
    dims = [vol.shape[2], vol.shape[1], vol.shape[0]]
    origin = np.array([-1.0, 0.5, 2.0], np.float32)
    spacing = np.array([0.5, 0.25, 1.0], np.float32)
    dmc, m, _ = gpu_run(vol.reshape(-1), dims, origin, spacing, iso, refinement, pad, **opts)
    ref, _ = oracle_for(vol.reshape(-1), dims, origin, spacing, iso, refinement, pad, **opts)
    assert_parity(dmc, m, ref)


@pytest.mark.parametrize("step", [0, 1, 2, 3, 4, 5, 6, STEP_ALL])
def test_splitting_steps_bit_exact(step):
    vol = np.random.default_rng(11).random((12, 12, 12), dtype=np.float32)
    dims = [12, 12, 12]
    o, s = np.zeros(3, np.float32), np.ones(3, np.float32)
    dmc, m, _ = gpu_run(vol.reshape(-1), dims, o, s, 0.5, 0, False, splitting_step=step)
    ref, _ = oracle_for(vol.reshape(-1), dims, o, s, 0.5, 0, False, splitting_step=step)
    assert_parity(dmc, m, ref)


def test_empty_and_degenerate_grids():
    o, s = np.zeros(3, np.float32), np.ones(3, np.float32)
    # nothing crosses the iso-value: the reference returns before post-processing
    dmc, m, _ = gpu_run(np.zeros(8 ** 3, np.float32), [8, 8, 8], o, s, 0.5)
    assert len(m.positions) == 0 and len(m.face_first_halfedge) == 0 and dmc.get_num_edges() == -1
    dmc, m, _ = gpu_run(np.ones(8 ** 3, np.float32), [8, 8, 8], o, s, 0.5)
    assert len(m.positions) == 0
    # a single cell
    v = np.array([0, 1, 0, 0, 0, 0, 0, 0], np.float32)
    dmc, m, _ = gpu_run(v, [2, 2, 2], o, s, 0.5)
    ref, _ = oracle_for(v, [2, 2, 2], o, s, 0.5)
    assert_parity(dmc, m, ref)
    assert len(m.positions) == 1 and len(m.face_first_halfedge) == 0
    # flat grids have no cells
    dmc, m, _ = gpu_run(np.random.default_rng(0).random(16, dtype=np.float32), [4, 4, 1], o, s, 0.5)
    assert len(m.positions) == 0


@pytest.mark.parametrize("which", [0, 1])
def test_reference_edge_case_grids(which):
    # generateEdgeCase, D/UniformGrid.inl:191-269 and :488-509: 4x4x3 grids of
    # 850/950 whose non-manifold vertex is detected without padding
    lo, hi = 850.0, 950.0
    v = np.full((3, 4, 4), lo, np.float32)
    v[0, 1, 2] = hi
    v[0, 2, 1] = hi
    if which == 1:
        v[1, 2, 1] = hi
    dims = [4, 4, 3]
    spacing = (np.float32(2.0) / (np.array(dims, np.float32) - np.float32(1))).astype(np.float32)
    origin = np.full(3, -1.0, np.float32)
    opts = dict(split_non_manifold=0)
    dmc, m, _ = gpu_run(v.reshape(-1), dims, origin, spacing, 900.0, **opts)
    ref, _ = oracle_for(v.reshape(-1), dims, origin, spacing, 900.0, **opts)
    assert_parity(dmc, m, ref)
    assert dmc.get_num_non_manifold_vertices() >= 1


def test_repeated_runs_reuse_context():
    vol = blobs(20, 5, 21)
    dims = [20, 20, 20]
    o, s = np.zeros(3, np.float32), np.ones(3, np.float32)
    dmc = mdmc.DualMarchingCubes()
    grid = mdmc.UniformGrid(vol, dims, o, s)
    dmc.run(0.5, grid)
    a = dmc.get_halfedge_mesh()
    big = mdmc.UniformGrid(np.random.default_rng(3).random((18, 18, 18), dtype=np.float32), [18, 18, 18], o, s)
    dmc.run(0.5, big)
    dmc.run(0.5, grid)
    b = dmc.get_halfedge_mesh()
    assert np.array_equal(a.halfedges, b.halfedges) and np.array_equal(a.positions, b.positions)


def test_write_obj_matches_reference_format(tmp_path):
    samples, dims, origin, spacing, iso = golden_grid("1-Edge")
    dmc, m, _ = gpu_run(samples, dims, origin, spacing, iso, 0, True)
    path = tmp_path / "m.obj"
    dmc.write_obj(path)
    lines = path.read_text().splitlines()
    v = [l for l in lines if l.startswith("v ")]
    f = [l for l in lines if l.startswith("f ")]
    assert len(v) == len(m.positions) and len(f) == len(m.quads)
    first = [int(t.split("//")[0]) - 1 for t in f[0].split()[1:]]
    assert first == list(m.quads[0])


@pytest.mark.parametrize("refinement,pad", [(0, True), (1, False), (2, False), (3, True)])
def test_materialized_refinement_bit_exact(refinement, pad):
    # the kernels read refined grids on demand; the dense form written by
    # mdmc_materialize_grid must equal refineGrid's output (oracle)
    import torch
    vol = blobs(11, 4, 31)
    dims = [11, 11, 11]
    origin = np.array([0.5, -2.0, 1.0], np.float32)
    spacing = np.array([0.3, 0.7, 1.1], np.float32)
    grid = mdmc.UniformGrid(vol, dims, origin, spacing, refinement, pad)
    out = torch.empty(grid.get_cell_count(), dtype=torch.float32, device="cuda")
    grid.materialize(out.data_ptr())
    torch.cuda.synchronize()
    ref, d, o, s = oracle_refine(vol.reshape(-1), dims, origin, spacing, refinement, pad)
    assert grid.dimensions == d
    assert np.array_equal(grid.origin, o) and np.array_equal(grid.deltas, s)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def _hsv(h, s=np.float32(0.8), v=np.float32(0.8)):
    # LazyEngine::Color::HSVtoRGB in float32
    f = np.float32(h) / np.float32(60.0)
    hi = np.floor(f)
    f = np.float32(f - hi)
    one = np.float32(1)
    p, q, t = v * (one - s), v * (one - s * f), v * (one - s * (one - f))
    return {0: (v, t, p), 6: (v, t, p), 1: (q, v, p), 2: (p, v, t), 3: (p, q, v), 4: (t, p, v)}.get(int(hi), (v, p, q))


def test_render_buffers_match_the_mesh():
    import torch
    # non-manifold edges and a non-manifold vertex left unrepaired: several flag colours
    samples, dims, origin, spacing, iso = golden_grid("Non-Manifold-Vertex")
    dmc, m, _ = gpu_run(samples, dims, origin, spacing, iso, 0, False, split_non_manifold=0)
    assert len(set(int(f) for f in m.vertex_flags)) > 1
    verts, idx = dmc.render_buffers()
    torch.cuda.synchronize()
    verts, idx = verts.cpu().numpy(), idx.cpu().numpy().view(np.uint32).reshape(-1, 6)
    q = m.quads.astype(np.uint32)
    assert np.array_equal(idx, np.stack([q[:, 0], q[:, 1], q[:, 2], q[:, 2], q[:, 3], q[:, 0]], 1))
    used = m.vertex_halfedge >= 0
    assert np.array_equal(verts[used, :3].view(np.uint32), m.positions[used].view(np.uint32))
    assert np.array_equal(verts[used, 3:6].view(np.uint32), m.normals[used].view(np.uint32))
    assert np.all(np.isnan(verts[~used, :6]))
    for v in np.flatnonzero(used):
        fl = int(m.vertex_flags[v])
        nm, weird, fans = fl & 1, fl & 4, fl & 8
        hue = 180.0
        if nm: hue = 0.0
        if weird: hue = 60.0
        if fans: hue = 270.0
        if weird and nm: hue = 300.0
        if nm and fans: hue = 240.0
        assert np.array_equal(verts[v, 6:9], np.array(_hsv(hue), np.float32)), (v, fl)
        assert verts[v, 9] == 1.0


def test_one_context_over_growing_and_shrinking_grids():
    """Buffers sized by earlier runs (the active-cell list is written during
    the scan when it already has room, after it otherwise) give the same
    meshes as a fresh context, on plain and refined grids."""
    o, s = np.zeros(3, np.float32), np.ones(3, np.float32)
    grids = [
        mdmc.UniformGrid(blobs(14, 3, 61), [14, 14, 14], o, s),
        mdmc.UniformGrid(np.random.default_rng(62).random((22, 22, 22), dtype=np.float32), [22, 22, 22], o, s),
        mdmc.UniformGrid(blobs(17, 5, 63), [17, 17, 17], o, s, 3, True),
        mdmc.UniformGrid(blobs(14, 3, 61), [14, 14, 14], o, s),
        mdmc.UniformGrid(np.random.default_rng(64).random((9, 12, 10), dtype=np.float32), [10, 12, 9], o, s, 1, False),
    ]
    isos = [0.5, 0.5, 0.4, 0.5, 0.5]
    shared = mdmc.DualMarchingCubes()
    for g, iso in zip(grids, isos):
        fresh = mdmc.DualMarchingCubes()
        fresh.run(iso, g)
        shared.run(iso, g)
        a, b = fresh.get_halfedge_mesh(), shared.get_halfedge_mesh()
        assert np.array_equal(a.halfedges, b.halfedges)
        assert np.array_equal(a.positions.view(np.uint32), b.positions.view(np.uint32))
        assert np.array_equal(a.vertex_flags, b.vertex_flags)
        assert fresh.stats.num_active_cells == shared.stats.num_active_cells
