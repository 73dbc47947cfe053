"""Timing is selected per item (mdmc_set_kernel_timing): selected kernels get
positive times, the others read 0, the stage times are on by default and can
be switched off, and timing changes no result."""
import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from manifolddmc_gb300.workloads import CONFIGS

pytestmark = pytest.mark.gpu


def _grid():
    desc, gen, iso, refine, pad = CONFIGS["blobs64_pad"]
    vol = gen()
    dims = [vol.shape[2], vol.shape[1], vol.shape[0]]
    return mdmc.UniformGrid(vol, dims, refinement=refine, add_zero_boundary=pad), iso


def test_kernel_timing_mask_selects_fields():
    grid, iso = _grid()
    dmc = mdmc.DualMarchingCubes()
    stages = dmc.run(iso, grid)
    assert stages["Total"] > 0 and stages["DMC"] > 0
    for _, field in mdmc.KERNEL_TIMING.values():
        assert getattr(dmc.stats, field) == 0.0
    base = dmc.get_halfedge_mesh()

    dmc.set_kernel_timing(["quads", "vertices"])
    dmc.run(iso, grid)
    assert dmc.stats.ms_quads > 0 and dmc.stats.ms_vertices > 0
    assert dmc.stats.ms_count == 0.0 and dmc.stats.ms_emit == 0.0

    dmc.set_kernel_timing(mdmc.TIME_ALL)
    dmc.run(iso, grid)
    for k in ("count", "emit", "quads", "vertices"):
        assert getattr(dmc.stats, mdmc.KERNEL_TIMING[k][1]) > 0, k
    timed = dmc.get_halfedge_mesh()
    for name in ("positions", "quads", "halfedges", "vertex_flags"):
        assert np.array_equal(np.asarray(getattr(base, name)).view(np.uint8), np.asarray(getattr(timed, name)).view(np.uint8)), name


def test_stage_timing_can_be_switched_off():
    grid, iso = _grid()
    dmc = mdmc.DualMarchingCubes()
    dmc.set_kernel_timing(["quads"], stages=False)
    stages = dmc.run(iso, grid)
    assert all(v == 0.0 for v in stages.values()), stages
    assert dmc.stats.ms_quads > 0
    dmc.set_kernel_timing([])
    assert dmc.run(iso, grid)["Total"] > 0 and dmc.stats.ms_quads == 0.0


def test_kernel_timing_rejects_unknown_bits():
    dmc = mdmc.DualMarchingCubes()
    with pytest.raises(mdmc.MDMCError):
        dmc.set_kernel_timing(128)


def test_fan_key_marks_wrap_around():
    """Fan detection marks its keys with a per-pass number (1..255) instead of
    clearing them every run; 300 runs on one context pass the wrap-around and
    must keep giving the first run's non-manifold vertices."""
    seen_nm = False
    for which in (0, 1):
        for pad in (False, True):
            vol, dims, origin, spacing = mdmc.generate_edge_case(which)
            grid = mdmc.UniformGrid(vol, dims, origin=origin, spacing=spacing, add_zero_boundary=pad)
            dmc = mdmc.DualMarchingCubes()
            dmc.run(900.0, grid)
            first = dmc.get_halfedge_mesh()
            nm = dmc.get_num_non_manifold_vertices()
            seen_nm = seen_nm or nm > 0
            for i in range(300):
                dmc.run(900.0, grid)
                assert dmc.get_num_non_manifold_vertices() == nm, (which, pad, i)
                if i % 50 == 49:
                    m = dmc.get_halfedge_mesh()
                    assert np.array_equal(m.vertex_flags, first.vertex_flags), (which, pad, i)
    assert seen_nm  # the path that marks fan keys ran
