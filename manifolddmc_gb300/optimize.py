"""Fitting a grid's iso-surface to a point cloud with the differentiable
path: Adam on the grid samples, one-sided Chamfer loss (mean over the mesh
vertices of the squared distance to the nearest target point), DMC forward and
the hand-written adjoint each step.  No counterpart in the reference."""
import time

import torch

from . import DualMarchingCubes, PointIndex
from .autograd import dual_marching_cubes


def chamfer_to_points(positions, points, index=None):
    """Mean over `positions` [V, 3] of the squared distance to the nearest of
    `points` [P, 3]; differentiable in `positions` (nearest points fixed).
    The nearest points come from a PointIndex over `points` (made here when
    `index` is None)."""
    if len(positions) == 0:
        return positions.sum()
    if index is None:
        index = PointIndex(points)
    with torch.no_grad():
        idx, _ = index.nearest(positions)
    return ((positions - points[idx]) ** 2).sum(dim=1).mean()


def fit_to_points(samples, points, iso=0.0, steps=200, lr=0.1, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0),
                  timing=None):
    """Adam on a copy of `samples` (CUDA float32 [Z, Y, X]) toward `points`
    (CUDA float32 [P, 3], same frame as the mesh).  Returns the fitted grid, the
    loss of every step and the wall time in seconds.  With a dict `timing`,
    CUDA events split each step into the DMC forward, the nearest-point search
    with the loss, and the backward (adjoint) with the Adam update; the dict
    gets their mean milliseconds."""
    grid = samples.detach().clone().requires_grad_(True)
    opt = torch.optim.Adam([grid], lr=lr)
    dmc = DualMarchingCubes(enable_surface_to_vertex_iteration=0)
    index = PointIndex(points)
    losses = []
    events = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if timing is not None else None
        if ev:
            ev[0].record()
        opt.zero_grad(set_to_none=True)
        pos, _ = dual_marching_cubes(grid, iso, dmc=dmc, origin=origin, spacing=spacing)
        if ev:
            ev[1].record()
        loss = chamfer_to_points(pos, points, index)
        if ev:
            ev[2].record()
        loss.backward()
        opt.step()
        if ev:
            ev[3].record()
            events.append(ev)
        losses.append(loss.detach())
    torch.cuda.synchronize()
    seconds = time.perf_counter() - t0
    if timing is not None and events:
        for k, (a, b) in {"forward_ms": (0, 1), "nearest_loss_ms": (1, 2), "backward_adam_ms": (2, 3)}.items():
            timing[k] = sum(e[a].elapsed_time(e[b]) for e in events) / len(events)
    return grid.detach(), [float(x) for x in losses], seconds
