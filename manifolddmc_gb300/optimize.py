"""Fitting a grid's iso-surface to a point cloud with the differentiable
path: Adam on the grid samples, one-sided Chamfer loss (mean over the mesh
vertices of the squared distance to the nearest target point), DMC forward and
the hand-written adjoint each step.  No counterpart in the reference."""
import time

import torch

from . import DualMarchingCubes
from .autograd import dual_marching_cubes


def chamfer_to_points(positions, points, chunk=1024):
    """Mean over `positions` [V, 3] of the squared distance to the nearest of
    `points` [P, 3]; differentiable in `positions` (nearest points fixed)."""
    if len(positions) == 0:
        return positions.sum()
    with torch.no_grad():
        idx = torch.empty(len(positions), dtype=torch.long, device=positions.device)
        for i in range(0, len(positions), chunk):
            idx[i:i + chunk] = torch.cdist(positions[i:i + chunk], points).argmin(dim=1)
    return ((positions - points[idx]) ** 2).sum(dim=1).mean()


def fit_to_points(samples, points, iso=0.0, steps=200, lr=0.1, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0)):
    """Adam on a copy of `samples` (CUDA float32 [Z, Y, X]) toward `points`
    (CUDA float32 [P, 3], same frame as the mesh).  Returns the fitted grid, the
    loss of every step and the wall time in seconds."""
    grid = samples.detach().clone().requires_grad_(True)
    opt = torch.optim.Adam([grid], lr=lr)
    dmc = DualMarchingCubes(enable_surface_to_vertex_iteration=0)
    losses = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        opt.zero_grad(set_to_none=True)
        pos, _ = dual_marching_cubes(grid, iso, dmc=dmc, origin=origin, spacing=spacing)
        loss = chamfer_to_points(pos, points)
        loss.backward()
        opt.step()
        losses.append(loss.detach())
    torch.cuda.synchronize()
    return grid.detach(), [float(x) for x in losses], time.perf_counter() - t0
