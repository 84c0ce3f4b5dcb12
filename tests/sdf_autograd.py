"""Test-only torch.autograd binding of the engine's TSDF sampling adjoint.

Forward calls vh_sdf_sample through the C ABI on CUDA tensors; backward is
the vector-Jacobian product grad_points = grad_phi[:, None] * d phi / d point
from the same call (the analytic gradient of trilinear interpolation)."""
import torch


class SdfSample(torch.autograd.Function):
    @staticmethod
    def forward(ctx, points, volume):
        phi, grad, valid = volume.sdf_sample(points.detach().contiguous())
        ctx.save_for_backward(grad)
        ctx.mark_non_differentiable(valid)
        return phi, valid

    @staticmethod
    def backward(ctx, grad_phi, _grad_valid):
        (grad,) = ctx.saved_tensors
        return grad_phi[:, None] * grad, None


def sdf_sample(points, volume):
    return SdfSample.apply(points, volume)
