"""Differentiation form: ray end states as a differentiable function of the
initial states and of every depth and current node.

`ray_endpoints` is a torch.autograd.Function over the library's hand-written
kernels (include/mantaray_gpu.h, mr_diff_*): its forward integrates the rays
with the reference's RK4 stepper and equations (grid lookups without the
reference's f32 casts, see csrc/diff.cu) and keeps a checkpoint every
`checkpoint_every` steps (sqrt(steps) by default); its backward is the
discrete adjoint, recomputing each segment from its checkpoint.  torch
provides the device memory and the autograd plumbing only.
"""

from __future__ import annotations

import ctypes
import math

from . import _native as N


def _torch():
    import torch

    return torch


def grid(nx, ny, x0, y0, dx, dy) -> N.DiffGrid:
    """A regular grid: points per axis, first axis values, spacing."""
    return N.DiffGrid(int(nx), int(ny), float(x0), float(y0), float(dx), float(dy))


def _precision(t) -> int:
    torch = _torch()
    if t.dtype == torch.float64:
        return 64
    if t.dtype == torch.float32:
        return 32
    raise TypeError("the differentiation form works in float64 or float32")


def _stream(t):
    torch = _torch()
    return torch.cuda.current_stream(t.device).cuda_stream


def _check_field(name, t, g):
    if t.shape != (g.ny, g.nx) or not t.is_contiguous() or not t.is_cuda:
        raise ValueError(f"{name} must be a contiguous CUDA tensor of shape (ny, nx) = "
                         f"({g.ny}, {g.nx})")


class _Endpoints:
    """Holder of the torch.autograd.Function (built lazily so importing this
    module does not import torch)."""

    fn = None

    @classmethod
    def get(cls):
        if cls.fn is not None:
            return cls.fn
        torch = _torch()

        class RayEndpoints(torch.autograd.Function):
            @staticmethod
            def forward(ctx, x0, y0, kx0, ky0, depth, u, v, bgrid, cgrid, dt, steps,
                        checkpoint_every):
                p = _precision(x0)
                n = x0.numel()
                _check_field("depth", depth, bgrid)
                _check_field("u", u, cgrid)
                _check_field("v", v, cgrid)
                ins = [t.contiguous() for t in (x0, y0, kx0, ky0)]
                n_ck = (steps + checkpoint_every - 1) // checkpoint_every if steps else 0
                ckpt = torch.empty((max(n_ck, 1), 4, n), dtype=x0.dtype, device=x0.device)
                end = torch.empty((4, n), dtype=x0.dtype, device=x0.device)
                status = torch.empty(n, dtype=torch.uint8, device=x0.device)
                N.check(N.load().mr_diff_forward(
                    p, ctypes.byref(bgrid), depth.data_ptr(), ctypes.byref(cgrid), u.data_ptr(),
                    v.data_ptr(), n, *[t.data_ptr() for t in ins], float(dt), int(steps),
                    int(checkpoint_every), ckpt.data_ptr(), end.data_ptr(), status.data_ptr(),
                    _stream(x0)))
                ctx.save_for_backward(*ins, depth, u, v, ckpt, status)
                ctx.grids = (bgrid, cgrid)
                ctx.args = (float(dt), int(steps), int(checkpoint_every))
                ctx.mark_non_differentiable(status)
                return end, status

            @staticmethod
            def backward(ctx, grad_end, _grad_status):
                x0, y0, kx0, ky0, depth, u, v, ckpt, status = ctx.saved_tensors
                bgrid, cgrid = ctx.grids
                dt, steps, every = ctx.args
                n = x0.numel()
                p = _precision(x0)
                grad_end = grad_end.contiguous().to(x0.dtype)
                seg = torch.empty((every, 16, n), dtype=x0.dtype, device=x0.device)
                g0 = torch.empty((4, n), dtype=x0.dtype, device=x0.device)
                gd = torch.empty((bgrid.ny, bgrid.nx), dtype=torch.float64, device=x0.device)
                gu = torch.empty((cgrid.ny, cgrid.nx), dtype=torch.float64, device=x0.device)
                gv = torch.empty((cgrid.ny, cgrid.nx), dtype=torch.float64, device=x0.device)
                N.check(N.load().mr_diff_backward(
                    p, ctypes.byref(bgrid), depth.data_ptr(), ctypes.byref(cgrid), u.data_ptr(),
                    v.data_ptr(), n, x0.data_ptr(), y0.data_ptr(), kx0.data_ptr(), ky0.data_ptr(),
                    dt, steps, every, ckpt.data_ptr(), status.data_ptr(), grad_end.data_ptr(),
                    seg.data_ptr(), g0.data_ptr(), gd.data_ptr(), gu.data_ptr(), gv.data_ptr(),
                    _stream(x0)))
                return (g0[0], g0[1], g0[2], g0[3], gd.to(depth.dtype), gu.to(u.dtype),
                        gv.to(v.dtype), None, None, None, None, None)

        cls.fn = RayEndpoints
        return cls.fn


def ray_endpoints(x0, y0, kx0, ky0, depth, u, v, bgrid, cgrid, dt, steps, checkpoint_every=None):
    """End states (4, n) = (x, y, kx, ky) after `steps` RK4 steps, and the
    per-ray status (1: the ray left a grid or met depth <= 0; its end state is
    NaN and it contributes no gradient).  Differentiable with respect to
    x0, y0, kx0, ky0 (shape (n,)) and depth (bgrid), u, v (cgrid), each a
    (ny, nx) CUDA tensor of the same dtype (float64 or float32)."""
    if checkpoint_every is None:
        checkpoint_every = max(1, int(math.ceil(math.sqrt(max(steps, 1)))))
    return _Endpoints.get().apply(x0, y0, kx0, ky0, depth, u, v, bgrid, cgrid, dt, steps,
                                  checkpoint_every)


def tangent(x0, y0, kx0, ky0, depth, u, v, bgrid, cgrid, dt, steps, dstate0=None, d_depth=None,
            d_u=None, d_v=None):
    """Forward-mode derivative: (end states, d end states, status) along the
    initial-state tangent dstate0 (4, n) and node tangents d_depth, d_u, d_v."""
    torch = _torch()
    n = x0.numel()
    p = _precision(x0)
    if dstate0 is None:
        dstate0 = torch.zeros((4, n), dtype=x0.dtype, device=x0.device)
    end = torch.empty((4, n), dtype=x0.dtype, device=x0.device)
    d_end = torch.empty((4, n), dtype=x0.dtype, device=x0.device)
    status = torch.empty(n, dtype=torch.uint8, device=x0.device)
    ptr = (lambda t: t.contiguous().data_ptr() if t is not None else None)
    N.check(N.load().mr_diff_tangent(
        p, ctypes.byref(bgrid), depth.data_ptr(), ctypes.byref(cgrid), u.data_ptr(), v.data_ptr(),
        n, x0.data_ptr(), y0.data_ptr(), kx0.data_ptr(), ky0.data_ptr(),
        dstate0.contiguous().data_ptr(), ptr(d_depth), ptr(d_u), ptr(d_v), float(dt), int(steps),
        end.data_ptr(), d_end.data_ptr(), status.data_ptr(), _stream(x0)))
    return end, d_end, status


def endpoint_loss(end, status, y_target, theta_target):
    """The differentiation case's loss: sum over rays that completed of
    (y_end - y*)^2 + (theta_end - theta*)^2, theta = atan2(ky, kx)."""
    torch = _torch()
    ok = status == 0
    theta = torch.atan2(end[3], end[2])
    dy = torch.where(ok, end[1] - y_target, torch.zeros_like(end[1]))
    dth = torch.where(ok, theta - theta_target, torch.zeros_like(theta))
    return (dy * dy + dth * dth).sum()
