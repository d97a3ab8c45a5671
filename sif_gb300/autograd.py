"""The CIC density contrast smoothed at a radius, as a differentiable torch
operation on the particle positions.

Forward: the deposit (sifg_cic_device), the contrast, the smoothing
(top-hat or Gaussian, with the CIC window correction) -- the fields the
exodus finder searches. Backward: the smoothing is self-adjoint (a real,
even filter between an R2C and a C2R), so the incoming gradient is smoothed
the same way and handed to the deposit's adjoint (sifg_contrast_vjp_device),
a CIC gather with one weight replaced by its derivative. float32 positions
run the float form, float64 the FP64 form.
"""
import torch

from . import device


class SmoothedContrast(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, z, n_grid, box, radius, filter="gaussian", window="full"):
        grid = device.cic(x, y, z, n_grid, box)
        device.density_contrast(grid)
        out = device.smooth(grid, n_grid, box, radius, filter=filter, window=window)
        ctx.save_for_backward(x, y, z)
        ctx.params = (n_grid, box, radius, filter, window)
        return out

    @staticmethod
    def backward(ctx, grad):
        x, y, z = ctx.saved_tensors
        n_grid, box, radius, filter, window = ctx.params
        g = device.smooth(grad.contiguous(), n_grid, box, radius, filter=filter, window=window)
        gx, gy, gz = device.contrast_vjp(x, y, z, n_grid, box, g)
        return gx, gy, gz, None, None, None, None, None


def smoothed_contrast(x, y, z, n_grid, box, radius, filter="gaussian", window="full"):
    """The smoothed density contrast (n_grid^3 values), differentiable in x, y, z."""
    return SmoothedContrast.apply(x, y, z, n_grid, box, radius, filter, window)
