"""The FP64 oracle of the differentiable path (surface iteration off),
checked against FP64 central finite differences: the gradient of
L = sum_o dL/dpos[o] . pos[parent(o)] with respect to the grid samples
(processed grid), and through refineGrid to the coarse samples.  These pin
the oracle the GPU adjoint is compared with."""
import numpy as np
import pytest

from _support import OracleRun, refine_backward, refine_f64, refined_geometry, sphere_sdf

H = 1e-4


def _loss(run, grid64, g):
    return float(np.sum(g * run.positions_f64(grid64)))


def _effective(run, dLdpos):
    g = np.zeros((run.num_dmc_vertices, 3))
    for o in range(run.num_vertices):
        p = o if o < run.num_dmc_vertices else run.parents[o]
        if 0 <= p < run.num_dmc_vertices:
            g[p] += dLdpos[o]
    return g


def _check_fd(grad, f, base, nodes):
    scale = max(1.0, float(np.abs(grad).max()))
    for i in nodes:
        gp = base.copy()
        gp[i] += H
        gm = base.copy()
        gm[i] -= H
        fd = (f(gp) - f(gm)) / (2 * H)
        assert abs(fd - grad[i]) <= 1e-5 * scale, (i, fd, grad[i])


def _nodes(run, dims, count, rng):
    # grid nodes at the corners of cells holding vertices, plus some others
    touched = set()
    X, Y = dims[0], dims[1]
    for c in run.cells[: min(len(run.cells), 400)]:
        for k in range(8):
            x, y, z = c[0] + (k & 1), c[1] + ((k >> 1) & 1), c[2] + ((k >> 2) & 1)
            touched.add(int((z * Y + y) * X + x))
    touched = sorted(touched)
    pick = list(rng.choice(touched, size=min(count, len(touched)), replace=False))
    pick += list(rng.integers(0, int(np.prod(dims)), size=10))
    return pick


@pytest.mark.parametrize("split", [0, 1])
def test_oracle_gradient_matches_central_differences(split):
    rng = np.random.default_rng(5)
    n = 20
    grid = sphere_sdf(n, 6.3) + 0.05 * rng.standard_normal((n, n, n)).astype(np.float32)
    dims = [n, n, n]
    origin, spacing = np.array([-2.0, 0.5, 1.0], np.float32), np.array([0.5, 0.25, 1.0], np.float32)
    with OracleRun(grid, dims, origin, spacing, 0.0, surface_iteration=0, split_non_manifold=split) as run:
        assert run.num_dmc_vertices > 100
        dL = rng.standard_normal((run.num_vertices, 3))
        g64 = grid.astype(np.float64).reshape(-1)
        grad = run.backward(g64, dL)
        geff = _effective(run, dL)
        _check_fd(grad, lambda gg: _loss(run, gg, geff), g64, _nodes(run, dims, 120, rng))


def test_oracle_split_vertices_pass_gradient_to_parents():
    # noise has non-manifold edges: the splitter appends vertices, each with a
    # parent DMC vertex that receives its gradient
    rng = np.random.default_rng(7)
    grid = rng.random((10, 10, 10), dtype=np.float32)
    with OracleRun(grid, [10, 10, 10], np.zeros(3, np.float32), np.ones(3, np.float32), 0.5,
                   surface_iteration=0) as run:
        assert run.num_vertices > run.num_dmc_vertices
        extra = run.parents[run.num_dmc_vertices:]
        assert np.all((extra >= 0) & (extra < run.num_dmc_vertices))
        assert np.array_equal(run.parents[: run.num_dmc_vertices], np.arange(run.num_dmc_vertices))
        dL = np.zeros((run.num_vertices, 3))
        dL[run.num_dmc_vertices:] = 1.0
        only_children = run.backward(grid.astype(np.float64), dL)
        dL2 = np.zeros((run.num_vertices, 3))
        np.add.at(dL2, extra, 1.0)
        direct = run.backward(grid.astype(np.float64), dL2)
        assert np.allclose(only_children, direct, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("refinement,pad", [(1, False), (2, True)])
def test_oracle_gradient_through_refinement(refinement, pad):
    rng = np.random.default_rng(9)
    n = 9
    coarse = sphere_sdf(n, 2.7) + 0.05 * rng.standard_normal((n, n, n)).astype(np.float32)
    dims = [n, n, n]
    od, sp, org = refined_geometry(dims, [1, 1, 1], [0, 0, 0], refinement, pad)
    fine32 = refine_f64(coarse, dims, refinement, pad).astype(np.float32)
    with OracleRun(fine32, od, org, sp, 0.0, surface_iteration=0) as run:
        dL = rng.standard_normal((run.num_vertices, 3))
        geff = _effective(run, dL)
        c64 = coarse.astype(np.float64).reshape(-1)
        grad_fine = run.backward(refine_f64(c64, dims, refinement, pad), dL)
        grad = refine_backward(grad_fine, dims, refinement, pad)
        f = lambda cc: _loss(run, refine_f64(cc, dims, refinement, pad), geff)
        nodes = list(rng.choice(np.flatnonzero(np.abs(grad) > 0), size=60, replace=False)) + [0, 5]
        _check_fd(grad, f, c64, nodes)


def test_oracle_gradient_on_the_differentiable_workload_1k_nodes():
    # the 128^3 signed distance to a sphere of radius 40 cells at iso 0 (the
    # differentiable form's grid): FP64 central differences (h = 1e-4) on 1000
    # random grid nodes, most of them at corners of cells holding vertices
    import sys
    sys.path.insert(0, str(__import__("pathlib").Path(__file__).resolve().parents[1]))
    from manifolddmc_gb300.workloads import CONFIGS
    desc, gen, iso, refine, pad = CONFIGS["sphere128_sdf"]
    vol = gen()
    n = vol.shape[0]
    dims = [n, n, n]
    rng = np.random.default_rng(123)
    with OracleRun(vol, dims, np.zeros(3, np.float32), np.ones(3, np.float32), iso, surface_iteration=0) as run:
        assert run.num_dmc_vertices > 10000
        dL = rng.standard_normal((run.num_vertices, 3))
        g64 = vol.astype(np.float64).reshape(-1)
        grad = run.backward(g64, dL)
        geff = _effective(run, dL)
        touched = np.flatnonzero(grad != 0)
        nodes = list(rng.choice(touched, size=900, replace=False)) + list(rng.integers(0, vol.size, size=100))
        _check_fd(grad, lambda gg: _loss(run, gg, geff), g64, nodes)
