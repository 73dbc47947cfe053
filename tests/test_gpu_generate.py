"""Volume generators against numpy float32 restatements of the reference's
expressions (UniformGrid.inl:20-269): bit-exact for the polynomial surfaces,
within 4e-6 of the value range for the cos-based ones (the device cosf and the
host cos differ in the last bits); the generated sphere meshes to a closed
manifold through the CLI."""
import json

import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from manifolddmc_gb300 import cli, meshtools

pytestmark = pytest.mark.gpu

f32 = np.float32


def _coords(dims):
    d = np.asarray(dims)
    sp = (f32(1) - f32(-1)) / (d.astype(np.float32) - f32(1))
    z, y, x = np.meshgrid(np.arange(d[2]), np.arange(d[1]), np.arange(d[0]), indexing="ij")
    return (f32(-1) + x.astype(f32) * sp[0], f32(-1) + y.astype(f32) * sp[1], f32(-1) + z.astype(f32) * sp[2]), sp


def _sq(v):
    return v * v


def _torus_h(x, y, z, c0, c1, c2, p0, p1):
    c, a = _sq(f32(p0)), _sq(f32(p1))
    X, Y, Z = _sq(x - f32(c0)), _sq(y - f32(c1)), _sq(z - f32(c2))
    return _sq(X + Y + Z + c - a) - f32(4) * c * (X + Y)


def _reference(name, x, y, z):
    if name == "sphere":
        return ((x * x + y * y + z * z).astype(np.float64) - 0.16).astype(f32)
    if name == "torus":
        return _torus_h(x, y, z, 0, 0, 0, 0.3, 0.15)
    if name == "two_holed_torus":
        return np.minimum(_torus_h(x, y, z, -0.38, 0, 0, 0.3, 0.15), _torus_h(x, y, z, 0.2, 0.38, 0, 0.3, 0.15))
    if name == "goursat":
        q = lambda v: v * v * v * v
        s = _sq(x) + _sq(y) + _sq(z)
        return q(x) + q(y) + q(z) + f32(-1) * s + f32(0) * s + f32(0.5)
    if name == "genus_two":
        X = f32(1) * (f32(4) * ((x + f32(1)) / f32(2)) - f32(2))
        Y = f32(1) * (f32(4) * ((y + f32(1)) / f32(2)) - f32(2))
        Z = f32(1) * (f32(4) * ((z + f32(1)) / f32(2)) - f32(2))
        t = f32(2) * Y * (Y * Y - f32(3) * X * X) * (f32(1) - Z * Z)
        t = t + (X * X + Y * Y) * (X * X + Y * Y)
        return t - (f32(9) * Z * Z - f32(1)) * (f32(1) - Z * Z)
    if name in ("iwp", "neovius", "pw_hybrid"):
        alpha = {"iwp": f32(5.01), "neovius": f32(1), "pw_hybrid": f32(1.01)}[name]
        arg = lambda v: (((alpha * (v + f32(1))).astype(np.float64)) * np.pi).astype(f32)
        cx, cy, cz = (np.cos(arg(v).astype(np.float64)) for v in (x, y, z))
        if name == "iwp":
            return cx * cy + cy * cz + cz * cx - cx * cy * cz
        if name == "neovius":
            return 3 * (cx + cy + cz) + 4 * cx * cy * cz
        return 4 * (cx * cy + cy * cz + cz * cx) - 3 * cx * cy * cz + 0.8
    raise KeyError(name)


@pytest.mark.parametrize("name", ["sphere", "torus", "two_holed_torus", "goursat", "genus_two"])
def test_polynomial_surfaces_bit_exact(name):
    dims = [21, 17, 13]
    vol, origin, spacing = mdmc.generate_volume(name, dims)
    (x, y, z), sp = _coords(dims)
    assert np.array_equal(spacing, sp) and np.all(origin == -1)
    ref = _reference(name, x, y, z)
    assert np.array_equal(vol.cpu().numpy().view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("name", ["iwp", "neovius", "pw_hybrid"])
def test_periodic_surfaces_close(name):
    dims = [24, 24, 24]
    vol, _, _ = mdmc.generate_volume(name, dims)
    (x, y, z), _ = _coords(dims)
    ref = _reference(name, x, y, z)
    v = vol.cpu().numpy()
    assert np.abs(v - ref).max() <= 4e-6 * max(1.0, np.abs(ref).max())


def test_edge_cases():
    for which in (0, 1):
        vol, dims, origin, spacing = mdmc.generate_edge_case(which)
        v = np.full((3, 4, 4), 850.0, np.float32)
        v[0, 1, 2] = v[0, 2, 1] = 950.0
        if which:
            v[1, 2, 1] = 950.0
        assert dims == [4, 4, 3] and np.array_equal(vol.cpu().numpy(), v)


def test_cli_generated_sphere_is_manifold(tmp_path, capsys):
    b, obj, st = tmp_path / "s.bin", tmp_path / "s.obj", tmp_path / "Statistics.json"
    assert cli.main(["generate", "sphere", "--dims", "40", "40", "40", "--bin", str(b)]) == 0
    # sphere value f*1000 + 1000: iso 1000 is the f = 0 surface
    assert cli.main(["run", str(b), "--iso", "1000", "--obj", str(obj), "--stats", str(st)]) == 0
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    pos, quads = meshtools.read_obj(obj)
    assert len(quads) == out["faces"] > 100
    rep = meshtools.manifold_report(quads, len(pos))
    assert rep["manifold"] and rep["edges_by_faces"] == {2: rep["edges"]}
    rec = json.loads("[" + st.read_text().rstrip().rstrip(",") + "]")[0]
    assert rec["quads"]["numQuads"] == len(quads) and rec["edges"]["4-Edges"] == 0


def test_cli_standard_mc_and_quality_of_a_generated_torus(tmp_path, capsys):
    b, obj, qb = tmp_path / "t.bin", tmp_path / "t.obj", tmp_path / "qualityMC.bin"
    assert cli.main(["generate", "torus", "--dims", "48", "48", "48", "--bin", str(b)]) == 0
    assert cli.main(["mc", str(b), "--iso", "1000", "--obj", str(obj), "--quality", str(qb)]) == 0
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    pos, tris = meshtools.read_obj(obj)
    assert tris.shape[1] == 3 and len(tris) == out["triangles"] > 100
    rep = meshtools.manifold_report(tris, len(pos))
    assert rep["manifold"] and rep["edges_by_faces"] == {2: rep["edges"]}
    # genus 1: V - E + F = 0
    assert len(pos) - rep["edges"] + len(tris) == 0
    q = meshtools.read_quality_bin(qb)
    assert len(q) == len(tris)
    # the quantised samples put some crossings on grid points: triangles whose
    # three vertices coincide have 0/0 quality (NaN, as in the reference)
    fin = np.isfinite(q)
    assert np.all((q[fin] >= 0) & (q[fin] <= 1.0 + 1e-6))
    t = tris[~fin]
    assert np.all((pos[t[:, 0]] == pos[t[:, 1]]) & (pos[t[:, 1]] == pos[t[:, 2]]))
    # DMC run with the 5-coloring and the quality of its quads' triangles
    qd, o2 = tmp_path / "qualityDMC.bin", tmp_path / "d.obj"
    assert cli.main(["run", str(b), "--iso", "1000", "--color-faces", "--quality", str(qd), "--obj", str(o2)]) == 0
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert len(meshtools.read_quality_bin(qd)) == 2 * out["faces"]
