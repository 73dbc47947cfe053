"""Differentiable Dual Marching Cubes for PyTorch (no counterpart in the
reference, which is not differentiable).

``dual_marching_cubes(samples, iso)`` runs the CUDA pipeline on a CUDA float32
grid and returns the mesh's vertex positions (differentiable with respect to
the grid samples) and its quads.  The topology is fixed by the forward run; the
backward pass is the library's adjoint kernel (``mdmc_backward``), which needs
the surface-to-vertex iteration off, so the function forces it off.
"""
import torch

from . import DualMarchingCubes, UniformGrid


class _DMCFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, samples, dmc, iso, origin, spacing, refinement, pad):
        if not samples.is_cuda or samples.dtype != torch.float32 or samples.dim() != 3:
            raise ValueError("samples must be a CUDA float32 tensor [Z, Y, X]")
        samples = samples.detach().contiguous()
        dims = [samples.shape[2], samples.shape[1], samples.shape[0]]
        stream = torch.cuda.current_stream()
        # A grid on the device only describes the samples' memory (refinement
        # and padding are evaluated from it on demand): the description of the
        # last call is reused when the samples sit at the same address with the
        # same layout (an optimiser updating them in place), which saves a
        # library context per step.
        key = (samples.data_ptr(), tuple(dims), tuple(origin), tuple(spacing), int(refinement), bool(pad))
        cached = getattr(dmc, "_grid_cache", None)
        if cached is not None and cached[0] == key:
            grid = cached[1]
        else:
            grid = UniformGrid(samples, dims, origin, spacing, refinement, pad, stream=stream)
            dmc._grid_cache = (key, grid)
        dmc.run(iso, grid, stream=stream)
        arrays = dmc.device_arrays(("positions", "quads"))
        positions = arrays["positions"].clone()
        quads = arrays["quads"].clone()
        ctx.mark_non_differentiable(quads)
        ctx.dmc = dmc
        ctx.grid = grid  # keeps the grid description (and its buffers) alive
        ctx.samples = samples
        ctx.run_id = dmc._run_id
        return positions, quads

    @staticmethod
    def backward(ctx, grad_positions, grad_quads):
        dmc = ctx.dmc
        if dmc._run_id != ctx.run_id:
            raise RuntimeError("the DualMarchingCubes object ran again after this forward; its topology is gone")
        out = torch.empty_like(ctx.samples)
        if grad_positions is None:
            out.zero_()
        else:
            dmc.backward(grad_positions.contiguous().float(), out, stream=torch.cuda.current_stream())
        return out, None, None, None, None, None, None


def dual_marching_cubes(samples, iso, dmc=None, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0), refinement=0,
                        pad=False):
    """Iso-surface of ``samples`` (CUDA float32 [Z, Y, X]) as ``(positions [V, 3], quads [F, 4])``.
    ``positions`` carries gradients back to ``samples``.  Pass a ``DualMarchingCubes``
    object to reuse its buffers; its surface iteration is switched off."""
    if dmc is None:
        dmc = DualMarchingCubes(enable_surface_to_vertex_iteration=0)
    elif dmc.options.enable_surface_to_vertex_iteration:
        dmc.set_option("enable_surface_to_vertex_iteration", 0)
    return _DMCFunction.apply(samples, dmc, float(iso), tuple(origin), tuple(spacing), int(refinement), bool(pad))
