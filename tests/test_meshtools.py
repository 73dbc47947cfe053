"""Host-side tooling: .bin round trip through the C ABI (host functions, no
GPU), OBJ canonical ordering, the manifold check and the statistics record."""
import json

import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from manifolddmc_gb300 import cli, meshtools
from _support import reference_goldens


def test_bin_round_trip(tmp_path):
    vol = (np.random.default_rng(0).random((5, 6, 7)) * 60000).astype(np.float32)
    path = tmp_path / "v.bin"
    mdmc.write_bin(path, vol, [0.5, 0.25, 2.0])
    back, dims, spacing, origin = mdmc.read_bin(path)
    assert dims == [7, 6, 5]
    assert np.array_equal(spacing, np.array([0.5, 0.25, 2.0], np.float32))
    assert np.array_equal(back, np.trunc(vol))  # uint16 storage truncates
    # origin = -(dims - 1) / 2 * spacing (UniformGrid.inl:563-566)
    assert np.allclose(origin, -(np.array(dims) - 1) / 2 * spacing)


def _golden(name, level):
    g = reference_goldens()[name]["levels"][str(level)]
    return np.asarray(g["v"], np.float32), np.asarray(g["f"], np.int64)


def test_canonical_form_ignores_order():
    pos, faces = _golden("Iterative-Fix", 3)
    rng = np.random.default_rng(1)
    perm = rng.permutation(len(pos))
    inv = np.argsort(perm)
    pos2 = pos[perm]
    faces2 = inv[faces][rng.permutation(len(faces))]
    faces2 = np.stack([np.roll(f, int(rng.integers(4))) for f in faces2])
    a = meshtools.canonicalize(pos, faces)
    b = meshtools.canonicalize(pos2, faces2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("name", ["1-Edge", "2-Edge", "3-Edge"])
def test_manifold_report_on_reference_meshes(name):
    # the unrepaired mesh has 4-face edges; the reference's fully split mesh has none
    rep0 = meshtools.manifold_report(_golden(name, 0)[1])
    rep3 = meshtools.manifold_report(_golden(name, 3)[1])
    assert rep0["edges_by_faces"].get(4, 0) > 0 and not rep0["manifold"]
    assert rep3["edges_by_faces"].get(4, 0) == 0


def test_cli_check_and_canonical(tmp_path, capsys):
    pos, faces = _golden("2-Edge", 3)
    src = tmp_path / "m.obj"
    meshtools.write_obj(src, pos, faces)
    assert cli.main(["check", str(src)]) == 0
    rep = json.loads(capsys.readouterr().out)
    assert rep["vertices"] == len(np.unique(faces))
    out = tmp_path / "c.obj"
    assert cli.main(["canonical", str(src), str(out)]) == 0
    p2, f2 = meshtools.read_obj(out)
    p1, f1 = meshtools.canonicalize(pos, faces)
    assert np.allclose(p2, p1) and np.array_equal(f2, f1)


def test_statistics_record_layout():
    class S:
        num_edges, num_edges3, num_edges4, num_non_manifold_vertices, num_dmc_quads = 10, 1, 2, 3, 4
        quads_with_non_manifold_edges = [5, 6, 7, 8]
    r = meshtools.statistics_record("a.bin", [3, 4, 5], 900.0, S, 11)
    assert r["numCells"] == 2 * 3 * 4
    assert list(r) == ["fileName", "dimensions", "numCells", "isoValue", "edges", "vertices", "quads"]
    assert r["quads"] == {"numQuads": 4, "1-Quads": 5, "2-Quads": 6, "3-Quads": 7, "4-Quads": 8}


def test_triangle_obj_and_quality_bin(tmp_path):
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    nrm = np.eye(4, 3, dtype=np.float32)
    tri = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]], np.int32)
    meshtools.write_triangle_obj(tmp_path / "t.obj", pos, nrm, tri)
    p2, f2 = meshtools.read_obj(tmp_path / "t.obj")
    assert np.array_equal(p2, pos) and np.array_equal(f2, tri)
    rep = meshtools.manifold_report(f2, len(p2))
    assert rep["manifold"] and rep["edges"] == 6 and rep["edges_by_faces"] == {2: 6}
    cp, cf = meshtools.canonicalize(p2, f2[::-1])
    assert cf.shape == (4, 3) and np.all(cf[:, 0] == cf.min(axis=1))
    q = np.array([0.5, 1.0, 0.25], np.float32)
    meshtools.write_quality_bin(tmp_path / "q.bin", q)
    raw = (tmp_path / "q.bin").read_bytes()
    assert len(raw) == 4 + 12 and np.frombuffer(raw[:4], np.int32)[0] == 3
    assert np.array_equal(meshtools.read_quality_bin(tmp_path / "q.bin"), q)
