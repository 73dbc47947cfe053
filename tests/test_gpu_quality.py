"""Face coloring, quad -> triangle split and mean-ratio quality through the C
ABI against the oracle: face attributes, triangles and qualities bit-exact."""
import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from _support import golden_grid, oracle_color_faces, oracle_mean_ratio, oracle_quads_to_triangles

pytestmark = pytest.mark.gpu


def _noise_run(seed, n, split):
    vol = np.random.default_rng(seed).random((n, n, n), dtype=np.float32)
    dmc = mdmc.DualMarchingCubes(split_non_manifold_halfedges=int(split))
    dmc.run(0.5, mdmc.UniformGrid(vol, [n, n, n]))
    return dmc


def _golden_run(case):
    samples, dims, origin, spacing, iso = golden_grid(case)
    dmc = mdmc.DualMarchingCubes()
    dmc.run(iso, mdmc.UniformGrid(samples.reshape(dims[2], dims[1], dims[0]), dims, origin, spacing, 0, True))
    return dmc


RUNS = [
    ("noise24_unsplit", lambda: _noise_run(5, 24, False)),
    ("noise24_split", lambda: _noise_run(6, 24, True)),
    ("noise64_unsplit", lambda: _noise_run(7, 64, False)),
    ("golden_4-Edge", lambda: _golden_run("4-Edge")),
    ("golden_12-Merge", lambda: _golden_run("12-Merge")),
]


@pytest.mark.parametrize("name,make", RUNS, ids=[r[0] for r in RUNS])
def test_color_faces_matches_oracle(name, make):
    import torch
    dmc = make()
    before = dmc.get_halfedge_mesh()
    dmc.color_faces()
    torch.cuda.synchronize()
    after = dmc.get_halfedge_mesh()
    expect = oracle_color_faces(before.halfedges, before.face_first_halfedge, before.face_attributes)
    assert np.array_equal(after.face_attributes, expect)
    assert np.array_equal(after.halfedges, before.halfedges)


@pytest.mark.parametrize("name,make", RUNS[:3], ids=[r[0] for r in RUNS[:3]])
def test_quads_to_triangles_and_quality_match_oracle(name, make):
    import torch
    dmc = make()
    m = dmc.get_halfedge_mesh()
    dev = dmc.device_arrays()
    tri = mdmc.quads_to_triangles(dev["quads"])
    q = mdmc.mean_ratio(dev["positions"], tri)
    torch.cuda.synchronize()
    rtri = oracle_quads_to_triangles(m.quads)
    assert np.array_equal(tri.cpu().numpy(), rtri)
    rq = oracle_mean_ratio(m.positions, rtri)
    assert np.array_equal(q.cpu().numpy().view(np.uint32), rq.view(np.uint32))


def test_quality_of_standard_mc_triangles():
    import torch
    n = 40
    vol = np.random.default_rng(8).random((n, n, n), dtype=np.float32)
    dmc = mdmc.DualMarchingCubes()
    pos, nrm, tri = dmc.run_standard_mc(0.5, mdmc.UniformGrid(vol, [n, n, n]))
    q = mdmc.mean_ratio(torch.from_numpy(pos).cuda(), torch.from_numpy(tri).cuda())
    rq = oracle_mean_ratio(pos, tri)
    assert np.array_equal(q.cpu().numpy().view(np.uint32), rq.view(np.uint32))
    assert float(q.min()) >= 0.0 and float(q.max()) <= 1.0 + 1e-6


def test_quality_rejects_out_of_range_ids():
    import torch
    pos = torch.zeros((3, 3), dtype=torch.float32, device="cuda")
    tri = torch.tensor([[0, 1, 2], [0, 1, 3]], dtype=torch.int32, device="cuda")
    with pytest.raises(mdmc.MDMCError):
        mdmc.mean_ratio(pos, tri)
