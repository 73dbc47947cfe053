"""mdmc_run_batch: every grid of a batch gives the mesh a single mdmc_run
gives (bit for bit), whatever number of concurrent workers runs it."""
import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from manifolddmc_gb300.workloads import batch_grids

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a.positions.view(np.uint32), b.positions.view(np.uint32))
    assert np.array_equal(a.normals.view(np.uint32), b.normals.view(np.uint32))
    assert np.array_equal(a.halfedges, b.halfedges)
    assert np.array_equal(a.face_first_halfedge, b.face_first_halfedge)
    assert np.array_equal(a.face_attributes, b.face_attributes)
    assert np.array_equal(a.vertex_flags, b.vertex_flags)


@pytest.mark.parametrize("streams", [0, 1, 3])
def test_batch_matches_single_runs(streams):
    items = batch_grids(count=10, seed=7, dim_range=(8, 40))
    grids = [mdmc.UniformGrid(vol) for vol, _ in items]
    isos = [iso for _, iso in items]
    batch = mdmc.BatchedDualMarchingCubes(streams=streams)
    stats = batch.run(grids, isos)
    assert batch.streams in ((1, 2, 4, 8, 16) if streams == 0 else (streams,))
    single = mdmc.DualMarchingCubes()
    for i, (g, iso) in enumerate(zip(grids, isos)):
        single.run(iso, g)
        assert int(stats[i].num_dmc_quads) == single.get_num_quads()
        assert int(stats[i].num_edges4) == single.get_num_non_manifold_edges4()
        _same(batch.get_halfedge_mesh(i), single.get_halfedge_mesh())
    # a second batch on the same object reuses its slots
    stats2 = batch.run(grids[:4], isos[:4])
    for i in range(4):
        assert int(stats2[i].num_dmc_vertices) == int(stats[i].num_dmc_vertices)


def test_full_batch_workload_matches_single_runs():
    """The bench's batch workload (96 grids, dims uniform in [24, 192], half
    Gaussian blobs and half uniform noise, iso in [0.3, 0.7]): every grid's
    mesh from one batch call equals a single mdmc_run's, bit for bit."""
    items = batch_grids()
    assert len(items) == 96
    grids = [mdmc.UniformGrid(vol) for vol, _ in items]
    isos = [iso for _, iso in items]
    batch = mdmc.BatchedDualMarchingCubes(streams=8)
    stats = batch.run(grids, isos)
    single = mdmc.DualMarchingCubes()
    splits = 0
    for i, (g, iso) in enumerate(zip(grids, isos)):
        single.run(iso, g)
        assert int(stats[i].num_dmc_quads) == single.get_num_quads()
        assert int(stats[i].num_non_manifold_vertices) == single.get_num_non_manifold_vertices()
        assert int(stats[i].split_iterations) == int(single.stats.split_iterations)
        splits += int(stats[i].split_iterations) > 0
        _same(batch.get_halfedge_mesh(i), single.get_halfedge_mesh())
    assert splits > 0  # the noise grids go through the splitter
