"""Test-only torch.autograd bindings of the engine's adjoints.

SdfSample: forward calls vh_sdf_sample through the C ABI on CUDA tensors;
backward is the vector-Jacobian product grad_points = grad_phi[:, None] *
d phi / d point from the same call (the analytic gradient of trilinear
interpolation).
IntegrateFrame: one integration update; backward is vh_integrate_vjp (the
update's VJP w.r.t. per-pixel depth and the se(3) pose)."""
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


def _se3_left(xi, pose):
    """exp(xi) * pose in FP64, xi = (v, w): the left perturbation of the
    engine's pose derivatives."""
    import numpy as np
    v, w = np.asarray(xi[:3], np.float64), np.asarray(xi[3:], np.float64)
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        R, V = np.eye(3) + K, np.eye(3) + 0.5 * K
    else:
        R = np.eye(3) + np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K
        V = np.eye(3) + (1 - np.cos(th)) / th ** 2 * K + (th - np.sin(th)) / th ** 3 * K @ K
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, V @ v
    return T @ np.asarray(pose, np.float64)


class IntegrateFrame(torch.autograd.Function):
    """One integration update as a differentiable function: from the volume
    state `pre` (exported blocks), integrate `depth` (H x W, metres) seen
    from exp(delta) * pose; the output is the sdf of the frame's blocks
    (n x 512), blocks sorted by their (x, y, z) coordinates (the block list's
    own order depends on GPU scheduling).  Backward calls vh_integrate_vjp, which
    recomputes the voxels' contributions from the volume (no tape), and
    returns dL/ddepth and dL/ddelta (at the perturbation's current value;
    the test evaluates it at delta = 0, where d pose / d delta is the left
    perturbation itself)."""

    @staticmethod
    def forward(ctx, depth, delta, volume, pose, rgb, pre):
        import numpy as np
        c2w = _se3_left(delta.detach().cpu().numpy(), pose).astype(np.float32)
        d = depth.detach().cpu().numpy().astype(np.float32)
        volume.reset()
        volume.import_blocks(pre["xyz"], pre["sdf"], pre["weight"], pre["rgb"])
        volume.integrate(d, rgb, c2w)
        lst = volume.block_list()
        order = np.lexsort(lst.T[::-1])
        e = volume.export_blocks()
        row = {tuple(k): i for i, k in enumerate(e["xyz"].tolist())}
        sdf = np.stack([e["sdf"][row[tuple(k)]] for k in lst[order].tolist()])
        ctx.volume, ctx.depth, ctx.c2w, ctx.order = volume, d, c2w, order
        return torch.from_numpy(sdf).to(depth.device)

    @staticmethod
    def backward(ctx, grad_sdf):
        import numpy as np
        g = np.empty(tuple(grad_sdf.shape), np.float32)
        g[ctx.order] = grad_sdf.detach().cpu().numpy()  # back to block-list order
        gd, gp = ctx.volume.integrate_vjp(ctx.depth, ctx.c2w, g)
        dev = grad_sdf.device
        return (torch.from_numpy(gd).to(dev), torch.from_numpy(gp).double().to(dev),
                None, None, None, None)


def integrate_frame(depth, delta, volume, pose, rgb, pre):
    return IntegrateFrame.apply(depth, delta, volume, pose, rgb, pre)
