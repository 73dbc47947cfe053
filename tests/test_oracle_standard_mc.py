"""The oracle's standard Marching Cubes (OriginalDMC standard_mc,
DualMarchingCubes.cu:201-328) on the CPU: its triangle table covers exactly
the intersected edges of every case (e_pattern, DualMarchingCubes.h:123), and
the meshes it makes of closed surfaces are closed, consistently oriented
2-manifolds with the Euler characteristic of their genus."""
import re

import numpy as np
import pytest

from _support import ORACLE_DIR, oracle_standard_mc, sphere_sdf

EDGE_V0 = [0, 1, 2, 0, 4, 5, 6, 4, 0, 1, 3, 2]
EDGE_AXIS = [0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2]


def _table():
    text = (ORACLE_DIR / "mc_triangle_table_oracle.h").read_text()
    start = text.index("kTriangleTable[256] = {")
    body = text[text.index("{", start) + 1:text.index("}", start)]
    return [int(v, 16) for v in re.findall(r"0x([0-9a-fA-F]+)ULL", body)]


def test_triangle_table_covers_exactly_the_intersected_edges():
    words = _table()
    assert len(words) == 256
    for cs, w in enumerate(words):
        n = w & 0xF
        used = {(w >> (4 + 4 * k)) & 0xF for k in range(3 * n)}
        crossing = set()
        for e in range(12):
            a0 = EDGE_V0[e]
            a1 = a0 | (1 << EDGE_AXIS[e])
            if ((cs >> a0) & 1) != ((cs >> a1) & 1):
                crossing.add(e)
        assert used == crossing, cs
        assert (n == 0) == (cs in (0, 255))


def _check_closed(pos, tri, genus):
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
    und = np.sort(e, axis=1)
    _, counts = np.unique(und, axis=0, return_counts=True)
    assert np.all(counts == 2)
    assert len(np.unique(e, axis=0)) == len(e)
    assert len(pos) - len(und) // 2 + len(tri) == 2 - 2 * genus


@pytest.mark.parametrize("n", [12, 21])
def test_oracle_standard_mc_closes_a_sphere(n):
    vol = sphere_sdf(n, 0.3 * n)
    pos, nrm, tri = oracle_standard_mc(vol, [n, n, n], np.zeros(3, np.float32), np.ones(3, np.float32), 0.0)
    _check_closed(pos, tri, 0)
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-5)
    c = (n - 1) / 2.0
    r = np.linalg.norm(pos - c, axis=1)
    assert np.all(np.abs(r - 0.3 * n) < 0.1)
    # normals of the distance field point outwards
    assert np.all(np.einsum("ij,ij->i", nrm, (pos - c) / r[:, None]) > 0.9)


def test_oracle_standard_mc_closes_a_torus():
    n = 32
    z, y, x = np.meshgrid(*(np.linspace(-1, 1, n),) * 3, indexing="ij")
    vol = ((np.sqrt(x * x + y * y) - 0.55) ** 2 + z * z - 0.2 ** 2).astype(np.float32)
    sp = np.float32(2.0 / (n - 1))
    pos, nrm, tri = oracle_standard_mc(vol, [n, n, n], np.full(3, -1, np.float32), np.full(3, sp, np.float32), 0.0)
    _check_closed(pos, tri, 1)


def test_oracle_standard_mc_without_cells_is_empty():
    vol = np.random.default_rng(0).random((1, 5, 6), dtype=np.float32)
    pos, nrm, tri = oracle_standard_mc(vol, [6, 5, 1], np.zeros(3, np.float32), np.ones(3, np.float32), 0.5)
    assert len(pos) == 0 and len(tri) == 0
