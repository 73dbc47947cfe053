"""The nearest-point index (mdmc_point_index_*, used by the Chamfer loss of
the differentiable workload, a tiled exhaustive GPU search) against a brute-force torch search with the same
float formula, (dx*dx + dy*dy) + dz*dz: the distance must be the exact
minimum and the index the smallest index attaining it."""
import numpy as np
import pytest

import manifolddmc_gb300 as mdmc
from manifolddmc_gb300.workloads import torus_points

pytestmark = pytest.mark.gpu


def brute_force(points, queries, chunk=512):
    import torch
    best_d = torch.empty(len(queries), dtype=torch.float32, device=queries.device)
    best_i = torch.empty(len(queries), dtype=torch.long, device=queries.device)
    idx = torch.arange(len(points), device=points.device)
    for s in range(0, len(queries), chunk):
        q = queries[s:s + chunk]
        d = q[:, None, :] - points[None, :, :]
        d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
        m = d2.min(dim=1).values
        best_d[s:s + chunk] = m
        # smallest index attaining the minimum
        cand = torch.where(d2 == m[:, None], idx[None, :], torch.full_like(d2, len(points), dtype=torch.long))
        best_i[s:s + chunk] = cand.min(dim=1).values
    return best_i, best_d


CASES = [
    ("uniform_box", lambda g: np.random.default_rng(g).uniform(-3, 5, (20000, 3))),
    ("torus", lambda g: torus_points(50000, 40.0, 15.0, (63.5, 63.5, 63.5), seed=g)),
    ("small_torus", lambda g: torus_points(20000, 10.0, 4.0, (0.0, 0.0, 0.0), seed=g)),
    ("on_a_lattice_with_ties", lambda g: np.stack(np.meshgrid(*[np.arange(12.0)] * 3), -1).reshape(-1, 3)),
    ("one_point", lambda g: np.array([[1.0, 2.0, 3.0]])),
    ("duplicates", lambda g: np.repeat(np.random.default_rng(g).uniform(0, 1, (50, 3)), 7, axis=0)),
    ("a_plane", lambda g: np.c_[np.random.default_rng(g).uniform(0, 9, (5000, 2)), np.zeros(5000)]),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_nearest_equals_brute_force(name, make):
    import torch
    pts = torch.from_numpy(np.asarray(make(7), np.float32)).cuda()
    lo, hi = pts.min(0).values, pts.max(0).values
    ext = (hi - lo).clamp(min=1.0)
    g = torch.Generator(device="cuda").manual_seed(11)
    # queries inside the box, around it, and on the lattice itself (exact ties)
    q = torch.rand((3000, 3), device="cuda", generator=g) * (1.6 * ext) + (lo - 0.3 * ext)
    q = torch.cat([q, pts[: min(len(pts), 500)] + 0.5, pts[: min(len(pts), 200)]])
    index = mdmc.PointIndex(pts)
    got_i, got_d = index.nearest(q)
    ref_i, ref_d = brute_force(pts, q)
    torch.cuda.synchronize()
    assert torch.equal(got_d, ref_d), (got_d - ref_d).abs().max()
    assert torch.equal(got_i, ref_i)
    assert len(index) == len(pts)


def test_chamfer_uses_exact_nearest_points():
    import torch
    from manifolddmc_gb300.optimize import chamfer_to_points
    pts = torch.from_numpy(torus_points(40000, 20.0, 7.0, (32.0, 32.0, 32.0), seed=2)).cuda()
    pos = (torch.rand((5000, 3), device="cuda") * 64.0).requires_grad_(True)
    loss = chamfer_to_points(pos, pts)
    _, ref_d = brute_force(pts, pos.detach())
    assert torch.allclose(loss.detach(), ref_d.mean(), rtol=1e-5)
    loss.backward()
    assert torch.isfinite(pos.grad).all()
