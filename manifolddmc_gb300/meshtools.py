"""Mesh tooling around the DMC path: OBJ reading, canonical ordering, a
manifold check and the reference GUI's statistics record.

- ``read_obj``: positions and faces (quads, or triangles) of an OBJ written
  by ``mdmc_write_obj`` or by the reference (Mesh::writeToFile,
  Mesh.cu:446-510: ``v``, ``vn`` and ``f a//a b//b c//c d//d`` lines,
  1-based).
- ``write_triangle_obj``: a triangle mesh with normals, ``f a//a b//b c//c``.
- ``write_quality_bin`` / ``read_quality_bin``: the element-quality file of
  the older CLI version (int32 count, then float32 per triangle;
  OriginalDMC/src/DualMarchingCubes.cu:909-916, 1015-1022).
- ``canonicalize``: vertices sorted by position (unreferenced ones dropped),
  each face rotated to start at its smallest vertex, faces sorted; two meshes
  with the same geometry and connectivity compare equal after it.
- ``manifold_report``: faces per edge (vertex pair) and fans per vertex.
- ``statistics_record``: the JSON object DMCImGui::writeMeshStatistics
  appends to Statistics.json (VisualDMC/src/LayerCUDA.cpp:638-676).
"""
import json

import numpy as np


def read_obj(path):
    pos, faces = [], []
    with open(path) as f:
        for line in f:
            if line.startswith("v "):
                pos.append([float(t) for t in line.split()[1:4]])
            elif line.startswith("f "):
                faces.append([int(t.split("/")[0]) - 1 for t in line.split()[1:]])
    width = len(faces[0]) if faces else 4
    return np.asarray(pos, np.float32).reshape(-1, 3), np.asarray(faces, np.int64).reshape(-1, width)


def write_obj(path, positions, faces):
    faces = np.asarray(faces)
    fmt = "f" + " %d" * (faces.shape[1] if faces.ndim == 2 else 4) + "\n"
    with open(path, "w") as f:
        for p in positions:
            f.write("v %.9g %.9g %.9g\n" % tuple(p))
        for q in faces:
            f.write(fmt % tuple(int(v) + 1 for v in q))


def write_triangle_obj(path, positions, normals, triangles):
    with open(path, "w") as f:
        for p in positions:
            f.write("v %.9g %.9g %.9g\n" % tuple(p))
        for n in normals:
            f.write("vn %.9g %.9g %.9g\n" % tuple(n))
        for t in triangles:
            a, b, c = (int(v) + 1 for v in t)
            f.write("f %d//%d %d//%d %d//%d\n" % (a, a, b, b, c, c))


def write_quality_bin(path, quality):
    q = np.ascontiguousarray(quality, np.float32)
    with open(path, "wb") as f:
        f.write(np.int32(len(q)).tobytes())
        f.write(q.tobytes())


def read_quality_bin(path):
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(4), np.int32)[0])
        return np.frombuffer(f.read(4 * n), np.float32).copy()


def canonicalize(positions, quads):
    """(positions, faces) in canonical order (quads or triangles)."""
    positions = np.asarray(positions, np.float32)
    quads = np.asarray(quads, np.int64)
    w = quads.shape[1] if quads.ndim == 2 else 4
    quads = quads.reshape(-1, w)
    used = np.unique(quads)
    order = used[np.lexsort(positions[used].T[::-1])]
    remap = np.full(len(positions), -1, np.int64)
    remap[order] = np.arange(len(order))
    q = remap[quads]
    start = np.argmin(q, axis=1)
    rot = np.stack([q[np.arange(len(q)), (start + k) % w] for k in range(w)], 1)
    rot = rot[np.lexsort(rot.T[::-1])]
    return positions[order], rot


def manifold_report(quads, num_vertices=None):
    """Counts of edges by face count, and of vertices with more than one fan
    (faces around a vertex connected through shared edges)."""
    quads = np.asarray(quads, np.int64)
    w = quads.shape[1] if quads.ndim == 2 else 4
    quads = quads.reshape(-1, w)
    n = int(num_vertices if num_vertices is not None else (quads.max() + 1 if len(quads) else 0))
    a = quads.reshape(-1)
    b = np.roll(quads, -1, axis=1).reshape(-1)
    key = np.minimum(a, b) * n + np.maximum(a, b)
    uniq, counts = np.unique(key, return_counts=True)
    hist = {int(k): int(v) for k, v in zip(*np.unique(counts, return_counts=True))}
    # fans: union-find of the faces around each vertex, joined across edges
    # that have exactly two faces
    face_of = np.repeat(np.arange(len(quads)), w)
    edge_faces = {}
    for k, f in zip(key.tolist(), face_of.tolist()):
        edge_faces.setdefault(k, []).append(f)
    parent = {}

    def find(x):
        while parent.get(x, x) != x:
            parent[x] = parent.get(parent[x], parent[x])
            x = parent[x]
        return x

    for k, fs in edge_faces.items():
        if len(fs) != 2:
            continue
        v0, v1 = divmod(k, n)
        for v in (v0, v1):
            ra, rb = find((v, fs[0])), find((v, fs[1]))
            if ra != rb:
                parent[ra] = rb
    fans = {}
    for f, q in enumerate(quads.tolist()):
        for v in set(q):
            fans.setdefault(v, set()).add(find((v, f)))
    multi = sum(1 for s in fans.values() if len(s) > 1)
    return {"edges": int(len(uniq)), "edges_by_faces": hist, "vertices": int(len(fans)),
            "multi_fan_vertices": int(multi),
            "manifold": bool(set(hist) <= {1, 2} and multi == 0)}


def statistics_record(file_name, dims, iso, stats, num_vertices):
    """DMCImGui::writeMeshStatistics's record (LayerCUDA.cpp:638-676)."""
    cells = (dims[0] - 1) * (dims[1] - 1) * (dims[2] - 1)
    q = stats.quads_with_non_manifold_edges
    return {"fileName": file_name, "dimensions": {"x": int(dims[0]), "y": int(dims[1]), "z": int(dims[2])},
            "numCells": int(cells), "isoValue": float(iso),
            "edges": {"numEdges": int(stats.num_edges), "3-Edges": int(stats.num_edges3),
                      "4-Edges": int(stats.num_edges4)},
            "vertices": {"numVertices": int(num_vertices), "nonManifoldVertices": int(stats.num_non_manifold_vertices)},
            "quads": {"numQuads": int(stats.num_dmc_quads), "1-Quads": int(q[0]), "2-Quads": int(q[1]),
                      "3-Quads": int(q[2]), "4-Quads": int(q[3])}}


def append_statistics(path, record):
    """Appends the record the way the reference does (an object followed by ',')."""
    with open(path, "a") as f:
        f.write(json.dumps(record, indent="\t") + ",\n")
