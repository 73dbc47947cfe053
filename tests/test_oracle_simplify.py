"""Invariants of the oracle's valence-pattern simplifications
(simplify3X3Y, simplify3X3YOld, simplify3333, HalfedgeMesh.cu:296-683 and
:859-1048).  The reference's test data holds no simplified meshes, so these
passes are pinned by invariants here and by GPU/oracle parity in
tests/test_gpu_parity.py: each removal keeps the Euler characteristic, every
pattern that was merged had the valences the reference requires, and the
rebuilt mesh references only existing vertices."""
import numpy as np
import pytest

from _support import oracle_run

from manifolddmc_gb300.workloads import gaussian_blobs

GRIDS = [
    ("noise16", lambda: np.random.default_rng(1).random((16, 16, 16), dtype=np.float32), 0.5),
    ("blobs32", lambda: gaussian_blobs(32, 6, (2.0, 5.0), 3), 0.4),
    ("blobs28_flat", lambda: gaussian_blobs(28, 3, (5.0, 9.0), 8), 0.3),
]
PASSES = [{"simplify_3x3y_color": 1}, {"simplify_3x3y_old": 1}, {"simplify_3333": 1},
          {"simplify_3x3y_color": 1, "simplify_3x3y_old": 1, "simplify_3333": 1}]


def _euler(r):
    return len(r["positions"]) - r["stats"]["edges"] + len(r["face_first"])


@pytest.mark.parametrize("name,factory,iso", GRIDS, ids=[g[0] for g in GRIDS])
def test_simplifications_keep_euler_characteristic(name, factory, iso):
    vol = factory()
    d = [vol.shape[2], vol.shape[1], vol.shape[0]]
    o, s = np.zeros(3, np.float32), np.ones(3, np.float32)
    base = oracle_run(vol.reshape(-1), d, o, s, iso, split_non_manifold=0, detect_non_manifold_vertices=0)
    reduced_any = False
    for opts in PASSES:
        r = oracle_run(vol.reshape(-1), d, o, s, iso, split_non_manifold=0, detect_non_manifold_vertices=0, **opts)
        assert r["stats"]["anomalies"] == 0
        assert _euler(r) == _euler(base), opts
        dv = len(base["positions"]) - len(r["positions"])
        df = len(base["face_first"]) - len(r["face_first"])
        assert dv == df >= 0, opts  # 3X3Y: one vertex and one quad per merge; 3333: four of each
        if "simplify_3333" in opts and len(opts) == 1:
            assert dv % 4 == 0
        reduced_any |= dv > 0
        he = r["halfedges"]
        assert he[:, 0].min() >= 0 and he[:, 0].max() < len(r["positions"])
        # the rebuilt mesh's twins pair up as the reference's initialize does
        tw = he[:, 3]
        paired = tw >= 0
        assert np.all(tw[paired] < len(he))
    assert reduced_any


def test_simplified_quads_lose_their_colour():
    vol = gaussian_blobs(32, 6, (2.0, 5.0), 3)
    d = [32, 32, 32]
    o, s = np.zeros(3, np.float32), np.ones(3, np.float32)
    r = oracle_run(vol.reshape(-1), d, o, s, 0.4, simplify_3x3y_color=1, split_non_manifold=0)
    # a rebuilt quad is a new QuadrilateralAttribute: INVALID_COLOR plus the NM/boundary bits
    assert np.all((r["face_attr"] & 0x1F) == 0x1F)
