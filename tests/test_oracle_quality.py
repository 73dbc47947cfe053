"""The oracle's consumers of the finished mesh from the older CLI version, on
the CPU: face coloring 24 -> 5 (FaceColoring.cu:5-141), quad -> triangle
split (DualMarchingCubes.cu:51-60) and mean-ratio quality
(QualityMeasure.h:45-66).

The coloring is pinned by a pure-Python restatement of the reference's
kernels run face by face (on a DMC mesh whose 24-coloring is proper, where
the reference's result does not depend on thread order), and by the
reference's own consistency check (checkFaceColoring,
DualMarchingCubes.cu:1055-1110): after the pass every face holds 0..4, and
the only neighbours that see each other and share a color are faces of
color 4 across the fourth edge, which the reference's test for color 4 skips
(:63).  (Across a four-face edge the twins need not be symmetric: a face can
border one that does not border it.)"""
import numpy as np
import pytest

from _support import (golden_grid, oracle_color_faces, oracle_mean_ratio, oracle_quads_to_triangles, oracle_refine,
                      oracle_run)


def _neighbour_faces(he, ff, f):
    out, e = [], ff[f]
    for _ in range(4):
        t = he[e, 3]
        out.append(he[t, 1] if t > -1 else -1)
        e = he[e, 2]
    return out


def _python_coloring(he, ff, attr):
    """color_faces / optimize_face_coloring, one face at a time, live reads."""
    col = [int(a) & 0x1F for a in attr]
    nb = [_neighbour_faces(he, ff, f) for f in range(len(ff))]

    def colors(f):
        return [col[g] if g > -1 else -1 for g in nb[f]]

    for cls in range(5, 24):
        for f in [f for f in range(len(ff)) if (attr[f] & 0x1F) == cls]:
            c0, c1, c2, c3 = colors(f)
            for k in range(4):
                if k not in (c0, c1, c2, c3):
                    col[f] = k
                    break
            else:
                if 4 not in (c0, c1, c2):
                    col[f] = 4
    for f in [f for f in range(len(ff)) if col[f] == 4]:
        c = colors(f)
        for k in range(4):
            if k not in c:
                col[f] = k
                break
    return col


def _unsplit_mesh(seed=3, n=14):
    g = np.random.default_rng(seed).random((n, n, n), dtype=np.float32)
    ref = oracle_run(g.reshape(-1), [n, n, n], np.zeros(3, np.float32), np.ones(3, np.float32), 0.5,
                     split_non_manifold=0)
    return ref["halfedges"].reshape(-1, 4), ref["face_first"], ref["face_attr"]


def _conflicts(he, ff, attr):
    out = []
    for f in range(len(ff)):
        for k, g in enumerate(_neighbour_faces(he, ff, f)):
            if g > -1 and (attr[g] & 0x1F) == (attr[f] & 0x1F):
                out.append((f, k, g))
    return out


def test_coloring_matches_python_restatement_and_the_reference_check():
    he, ff, attr = _unsplit_mesh()
    assert _conflicts(he, ff, attr) == []  # the DMC's grid-edge coloring is proper
    new = oracle_color_faces(he, ff, attr)
    assert [int(a) & 0x1F for a in new] == _python_coloring(he, ff, attr)
    assert np.array_equal(new & ~np.uint16(0x1F), attr & ~np.uint16(0x1F))
    assert (new & 0x1F).max() <= 4
    for f, k, g in _conflicts(he, ff, new):
        back = _neighbour_faces(he, ff, g)
        if f not in back:
            continue  # g does not see f: twins of a four-face edge are not symmetric
        # two faces of color 4, across the fourth edge of one of them
        assert (new[f] & 0x1F) == 4
        assert k == 3 or back.index(f) == 3


@pytest.mark.parametrize("case", ["4-Edge", "Iterative-Fix", "12-Merge"])
def test_coloring_of_repaired_golden_meshes(case):
    samples, dims, origin, spacing, iso = golden_grid(case)
    g, d, o, s = oracle_refine(samples, dims, origin, spacing, 0, True)
    ref = oracle_run(g, d, o, s, iso)
    he, ff, attr = ref["halfedges"].reshape(-1, 4), ref["face_first"], ref["face_attr"]
    new = oracle_color_faces(he, ff, attr)
    assert np.array_equal(new & ~np.uint16(0x1F), attr & ~np.uint16(0x1F))
    # every face of classes 0..23 ends in 0..4 on these meshes; the faces the
    # splitter made carry the invalid color 31, which no pass touches
    before, after = attr & 0x1F, new & 0x1F
    assert np.all(after[before < 24] <= 4)
    assert np.array_equal(after[before >= 24], before[before >= 24])


def test_quads_to_triangles_split():
    q = np.array([[0, 1, 2, 3], [4, 5, 6, 7]], np.int32)
    t = oracle_quads_to_triangles(q)
    assert t.tolist() == [[0, 1, 3], [3, 2, 0], [4, 5, 7], [7, 6, 4]]


def test_mean_ratio_known_values():
    s3 = np.sqrt(3.0)
    pos = np.array([[0, 0, 0], [1, 0, 0], [0.5, s3 / 2, 0], [0, 1, 0], [2, 0, 0], [0, 0, 3]], np.float32)
    tri = np.array([[0, 1, 2], [0, 1, 3], [0, 1, 4], [0, 3, 5]], np.int32)
    q = oracle_mean_ratio(pos, tri)
    p = pos.astype(np.float64)
    expect = []
    for a, b, c in tri:
        cr = np.linalg.norm(np.cross(p[b] - p[a], p[c] - p[a]))
        l = ((p[b] - p[a]) ** 2).sum() + ((p[c] - p[b]) ** 2).sum() + ((p[a] - p[c]) ** 2).sum()
        expect.append(2 * s3 * cr / l)
    assert np.allclose(q, expect, rtol=1e-6, atol=0)
    assert abs(q[0] - 1.0) < 1e-6 and q[2] == 0.0
