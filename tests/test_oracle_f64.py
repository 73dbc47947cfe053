"""The oracle's FP64 build (the same restatement compiled with
MDMC_ORACLE_REAL=double; bench.py times it as the CPU baseline) against the
float restatement: on the reference's golden grids and a refined blob grid
it must give the same mesh topology with positions within 1e-5 of the grid
spacing (or 8 float ulps of the largest coordinate, where that is coarser), and the one-call refine + run of the float build must equal the two
separate calls bit for bit."""
import numpy as np
import pytest

from _support import (LEVEL_OPTIONS, golden_grid, oracle_refine, oracle_run, oracle_run_refined,
                      reference_goldens)
from manifolddmc_gb300.workloads import gaussian_blobs


def _same_topology(a, b):
    assert a["halfedges"].shape == b["halfedges"].shape
    assert np.array_equal(a["halfedges"], b["halfedges"])
    assert np.array_equal(a["face_first"], b["face_first"])
    assert a["stats"] == b["stats"]


@pytest.mark.parametrize("case", list(reference_goldens().keys()))
@pytest.mark.parametrize("level", [0, 3])
def test_f64_build_matches_the_float_restatement_on_the_goldens(case, level):
    samples, dims, origin, spacing, iso = golden_grid(case)
    pad, opts = LEVEL_OPTIONS[level]
    f32 = oracle_run_refined(samples, dims, origin, spacing, 0, pad, iso, **opts)
    f64 = oracle_run_refined(samples, dims, origin, spacing, 0, pad, iso, f64=True, **opts)
    _same_topology(f32, f64)
    tol = 1e-5 * float(np.max(spacing))
    assert np.max(np.abs(f32["positions"] - f64["positions"])) <= tol


def test_f64_build_on_a_refined_blob_grid():
    v = gaussian_blobs(33, 8, (2.0, 6.0), 3)
    o, s = np.zeros(3, np.float32), np.ones(3, np.float32)
    f32 = oracle_run_refined(v, [33, 33, 33], o, s, 3, True, 0.4)
    f64 = oracle_run_refined(v, [33, 33, 33], o, s, 3, True, 0.4, f64=True)
    _same_topology(f32, f64)
    assert len(f32["positions"]) > 1000
    # coordinates reach 32 here, where one float ulp is 3.8e-6 (1.5e-5 of the
    # 0.25 spacing): the bound is 8 ulps of the largest coordinate
    ulp = np.spacing(np.float32(np.max(np.abs(f32["positions"]))))
    assert np.max(np.abs(f32["positions"] - f64["positions"])) <= 8 * ulp


def test_refined_run_in_one_call_equals_refine_then_run():
    v = gaussian_blobs(21, 5, (2.0, 5.0), 4)
    o, s = np.asarray([0.5, -1.0, 2.0], np.float32), np.asarray([0.25, 0.5, 1.0], np.float32)
    g, d, oo, ss = oracle_refine(v, [21, 21, 21], o, s, 2, True)
    two = oracle_run(g, d, oo, ss, 0.45)
    one = oracle_run_refined(v, [21, 21, 21], o, s, 2, True, 0.45)
    for k in two:
        if k == "stats":
            assert one[k] == two[k]
        else:
            assert np.array_equal(np.asarray(one[k]).view(np.uint8), np.asarray(two[k]).view(np.uint8)), k
