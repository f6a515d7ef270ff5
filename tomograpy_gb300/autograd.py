"""The projector as a differentiable torch operation.

``project(x, op)`` is y = P x with a hand-written backward: dL/dx = P^T dL/dy,
i.e. the backprojector kernel (and ``backproject`` the reverse), so
regularised reconstructions get exact gradients of their data term without
materialising the system matrix.  ``op`` is a device-resident
:class:`tomograpy_gb300.lo_wrapper.Siddon`.

``reconstruct_lbfgs`` is the differentiable-reconstruction workload:
minimise 1/2 ||P softplus(z) - y||^2 + tv * TV_eps(softplus(z)) with L-BFGS
(positivity by the softplus reparametrisation, smoothed total variation
TV_eps(x) = sum sqrt(|grad x|^2 + eps)).
"""
import torch


class _Project(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op):
        ctx.op = op
        return op.project(x.detach())

    @staticmethod
    def backward(ctx, gy):
        return ctx.op.backproject(gy.contiguous()), None


class _Backproject(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y, op):
        ctx.op = op
        return op.backproject(y.detach())

    @staticmethod
    def backward(ctx, gx):
        return ctx.op.project(gx.contiguous()), None


def project(x, op):
    """Differentiable y = P x."""
    return _Project.apply(x, op)


def backproject(y, op):
    """Differentiable x = P^T y."""
    return _Backproject.apply(y, op)


class SiddonProjector(torch.nn.Module):
    """nn.Module wrapper around a device-resident projector operator."""

    def __init__(self, op):
        super().__init__()
        self.op = op

    def forward(self, x):
        return project(x, self.op)


def tv_smooth(x, eps=1e-6):
    """Smoothed isotropic total variation of a 3-D cube (forward differences)."""
    gx = torch.diff(x, dim=0)[:, :-1, :-1]
    gy = torch.diff(x, dim=1)[:-1, :, :-1]
    gz = torch.diff(x, dim=2)[:-1, :-1, :]
    return torch.sqrt(gx * gx + gy * gy + gz * gz + eps).sum()


def reconstruct_lbfgs(op, y, iters=50, tv=1e-3, eps=1e-6, z0=None, scale=None, history_size=10):
    """L-BFGS reconstruction with positivity (softplus) and smoothed TV.

    ``scale`` rescales the unknowns (x = scale * softplus(z)) so that the
    optimiser works with O(1) numbers; by default it is max|y| / max chord.
    Returns (x, losses).
    """
    dev = y.device
    if scale is None:
        chord = 3.0 ** 0.5 * 3.0
        scale = float(y.abs().max()) / chord if float(y.abs().max()) > 0 else 1.0
    z = torch.zeros(op.cube_shape, dtype=torch.float32, device=dev) if z0 is None else z0.clone()
    z.requires_grad_(True)
    opt = torch.optim.LBFGS([z], lr=1.0, max_iter=iters, history_size=history_size,
                            line_search_fn="strong_wolfe", tolerance_grad=0.0, tolerance_change=0.0)
    losses = []
    norm = float((y.double() ** 2).sum()) or 1.0

    def closure():
        opt.zero_grad()
        x = scale * torch.nn.functional.softplus(z)
        r = project(x, op) - y
        loss = 0.5 * (r.double() ** 2).sum() / norm + tv * tv_smooth(x / scale, eps).double() / x.numel()
        loss.backward()
        losses.append(float(loss.detach()))
        return loss

    opt.step(closure)
    with torch.no_grad():
        x = scale * torch.nn.functional.softplus(z)
    return x.detach(), losses
