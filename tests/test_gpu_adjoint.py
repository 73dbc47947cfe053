"""The adjoint kernel (mdmc_backward) against the FP64 oracle gradient, which
tests/test_adjoint_oracle.py pins to FP64 central differences.  Tolerance:
max |gpu - fp64| <= 1e-5 * max |fp64| over all samples (float32 arithmetic,
float atomics).  The forward runs with the surface iteration off."""
import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from _support import OracleRun, oracle_refine, refine_backward, refined_geometry, sphere_sdf

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _blobs(n, count, seed):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    v = np.zeros((n, n, n))
    for _ in range(count):
        c = rng.uniform(0, n - 1, 3)
        s = rng.uniform(1.5, 4.0)
        v += np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    return v.astype(np.float32)


CASES = [
    # name, volume, iso, refinement, pad
    ("sphere24", lambda: sphere_sdf(24, 7.5) + 0.03 * np.random.default_rng(1).standard_normal((24,) * 3).astype(np.float32), 0.0, 0, False),
    ("noise12_split", lambda: np.random.default_rng(2).random((12, 12, 12), dtype=np.float32), 0.5, 0, False),
    ("blobs16_pad", lambda: _blobs(16, 5, 3), 0.4, 0, True),
    ("blobs9_refine3", lambda: _blobs(9, 4, 4), 0.35, 3, False),
    ("blobs8_refine1_pad", lambda: _blobs(8, 3, 5), 0.3, 1, True),
]


@pytest.mark.parametrize("name,factory,iso,refinement,pad", CASES, ids=[c[0] for c in CASES])
def test_backward_matches_fp64_oracle(name, factory, iso, refinement, pad):
    _check_backward(name, factory(), iso, refinement, pad)


def _sweep(n=16, seed=31):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = [int(rng.integers(3, 15)) for _ in range(3)]
        kind = "noise" if i % 2 else "blobs"
        out.append(("%02d_%s_%dx%dx%d" % (i, kind, *dims), kind, dims, int(rng.integers(0, 2**31)),
                    int(rng.choice([0, 1, 2, 3])), bool(rng.integers(0, 2))))
    return out


SWEEP = _sweep()


@pytest.mark.parametrize("name,kind,dims,seed,refinement,pad", SWEEP, ids=[c[0] for c in SWEEP])
def test_backward_sweep(name, kind, dims, seed, refinement, pad):
    rng = np.random.default_rng(seed)
    shape = (dims[2], dims[1], dims[0])
    if kind == "noise":
        vol, iso = rng.random(shape, dtype=np.float32), 0.5
    else:
        vol, iso = _blobs(max(dims), 3, seed % 1000)[:dims[2], :dims[1], :dims[0]].copy(), 0.3
    if not ((vol >= iso).any() and (vol < iso).any()):
        pytest.skip("no crossing in this field")
    _check_backward(name, vol, iso, refinement, pad, need_vertices=False)


def _check_backward(name, vol, iso, refinement, pad, need_vertices=True):
    torch = pytest.importorskip("torch")
    dims = [vol.shape[2], vol.shape[1], vol.shape[0]]
    origin = np.array([0.5, -1.0, 2.0], np.float32)
    spacing = np.array([0.25, 0.5, 1.0], np.float32)
    dmc = mdmc.DualMarchingCubes(enable_surface_to_vertex_iteration=0)
    samples = torch.from_numpy(vol).cuda()
    grid = mdmc.UniformGrid(samples, dims, origin, spacing, refinement, pad)
    dmc.run(iso, grid)
    V = int(dmc.mesh.num_vertices)
    if V == 0 and not need_vertices:
        return
    assert V > 0
    rng = np.random.default_rng(17)
    dl = rng.standard_normal((V, 3)).astype(np.float32)
    out = torch.full(vol.shape, 123.0, device="cuda")
    dmc.backward(torch.from_numpy(dl).cuda(), out)
    torch.cuda.synchronize()
    gpu = out.cpu().numpy().reshape(-1).astype(np.float64)

    fine, fd, fo, fs = oracle_refine(vol.reshape(-1), dims, origin, spacing, refinement, pad)
    with OracleRun(fine, fd, fo, fs, iso, surface_iteration=0) as run:
        assert run.num_vertices == V
        # the forward is the oracle's bit for bit (positions of the same topology)
        pos = dmc.device_arrays()["positions"].cpu().numpy()
        assert np.array_equal(pos.view(np.uint32), run.positions.view(np.uint32))
        ref = run.backward(fine.astype(np.float64), dl.astype(np.float64))
    if refinement or pad:
        ref = refine_backward(ref, dims, refinement, pad)
    scale = np.abs(ref).max()
    assert scale > 0
    err = np.abs(gpu - ref).max()
    assert err <= TOL * scale, (err, scale)
    if name == "noise12_split":
        assert V > dmc.get_num_vertices()  # split vertices passed their gradient on

    # accumulate adds to the buffer
    dmc.backward(torch.from_numpy(dl).cuda(), out, accumulate=True)
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy().reshape(-1) - 2 * ref).max() <= 2 * TOL * scale


def test_backward_needs_surface_iteration_off():
    torch = pytest.importorskip("torch")
    vol = sphere_sdf(12, 3.3)
    dmc = mdmc.DualMarchingCubes()
    dmc.run(0.0, mdmc.UniformGrid(vol))
    V = int(dmc.mesh.num_vertices)
    with pytest.raises(mdmc.MDMCError):
        dmc.backward(torch.zeros((V, 3), device="cuda"), torch.zeros(vol.shape, device="cuda"))


def test_autograd_function_and_optimisation_step():
    torch = pytest.importorskip("torch")
    from manifolddmc_gb300.autograd import dual_marching_cubes
    n = 32
    grid = torch.from_numpy(sphere_sdf(n, 9.0)).cuda().requires_grad_(True)
    pos, quads = dual_marching_cubes(grid, 0.0)
    assert pos.requires_grad and quads.dtype == torch.int32 and len(quads) > 0
    # pull every vertex toward the centre: raising the SDF near the surface
    # moves the surface inward, so d(loss)/d(sample) is mostly negative
    c = (n - 1) / 2.0
    loss = ((pos - c) ** 2).sum()
    loss.backward()
    g = grid.grad
    assert torch.isfinite(g).all() and g.abs().max() > 0
    assert (g < 0).sum() > 10 * (g > 0).sum()
    # a few Adam steps reduce the loss
    opt = torch.optim.Adam([grid], lr=0.05)
    dmc = None
    losses = []
    from manifolddmc_gb300 import DualMarchingCubes
    dmc = DualMarchingCubes(enable_surface_to_vertex_iteration=0)
    for _ in range(10):
        opt.zero_grad()
        pos, _ = dual_marching_cubes(grid, 0.0, dmc=dmc)
        loss = ((pos - c) ** 2).sum(dim=1).mean()
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert losses[-1] < losses[0]


def test_fit_sphere_to_torus_points():
    # the differentiable workload at a smaller size: a 48^3 sphere SDF pulled
    # toward points on a torus by Adam through forward + adjoint
    torch = pytest.importorskip("torch")
    from manifolddmc_gb300.optimize import fit_to_points
    from manifolddmc_gb300.workloads import sphere_sdf, torus_points
    n = 48
    c = (n - 1) / 2.0
    grid0 = torch.from_numpy(sphere_sdf(n, 15.0)).cuda()
    pts = torch.from_numpy(torus_points(20000, 15.0, 6.0, (c, c, c), seed=3)).cuda()
    _, losses, seconds = fit_to_points(grid0, pts, steps=30, lr=0.1)
    assert all(np.isfinite(losses))
    assert np.mean(losses[-5:]) < 0.9 * np.mean(losses[:5]), losses[::5]


def test_fit_full_size_differentiable_workload():
    """The differentiable workload at its full size: the 128^3 signed distance
    to a sphere of radius 40 cells pulled toward 200k points on a torus
    (R = 40, r = 15 cells) by 200 Adam steps of DMC forward + adjoint with the
    one-sided Chamfer loss (nearest points from the library's point index)."""
    torch = pytest.importorskip("torch")
    from manifolddmc_gb300.optimize import fit_to_points
    from manifolddmc_gb300.workloads import CONFIGS, torus_points
    desc, gen, iso, refine, pad = CONFIGS["sphere128_sdf"]
    vol = gen()
    c = (vol.shape[0] - 1) / 2.0
    grid0 = torch.from_numpy(vol).cuda()
    pts = torch.from_numpy(torus_points(200000, 40.0, 15.0, (c, c, c), seed=5)).cuda()
    fitted, losses, seconds = fit_to_points(grid0, pts, iso, steps=200, lr=0.1)
    assert all(np.isfinite(losses))
    # the surface moves about a cell per ten steps at lr 0.1 (only grid nodes at
    # crossing edges receive gradients), so 200 steps close part of the gap
    assert np.mean(losses[-10:]) < 0.97 * np.mean(losses[:10]), losses[::20]
    assert losses[-1] < losses[0]
    assert torch.isfinite(fitted).all()

