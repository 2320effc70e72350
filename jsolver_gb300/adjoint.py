"""Reverse-mode differentiation of the fixed-mode 2D solve (torch.autograd).

The reference differentiates ``solve_2d(..., fixed=True)`` with ``jax.vjp``
(jsolver/solver_2d.py:18-26; README: reverse mode works in fixed mode only). Here the
vector-Jacobian product is the hand-written adjoint in libjmg (``jmg_solve_fixed_vjp``:
transposed smoother, restriction and prolongation swapped, per-cycle checkpointing with
recomputation, backward of the coefficient hierarchy). ``solve_2d`` routes CUDA tensors
that require grad through ``FixedSolve2D`` when ``fixed=True``.
"""
import ctypes

import torch

from . import _engine, _lib


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


class FixedSolve2D(torch.autograd.Function):
    """phi_n = solve_2d(grid_x, grid_y, phi0, rhs, lam, D_xx, D_yy, fixed=True, ...)."""

    @staticmethod
    def forward(ctx, phi0, rhs, lam, D_xx, D_yy, grids, opts):
        shape = phi0.shape
        lam_a = lam.expand(shape).contiguous() if lam.dim() == 0 else lam.contiguous()
        Dx = D_xx.expand(shape).contiguous() if D_xx.dim() == 0 else D_xx.contiguous()
        Dy = D_yy.expand(shape).contiguous() if D_yy.dim() == 0 else D_yy.contiguous()
        phi0 = phi0.contiguous()
        rhs = rhs.contiguous()
        with torch.no_grad():
            phi, _ = _engine.solve(grids, phi0, rhs, lam_a, (Dx, Dy), None, **opts)
        ctx.save_for_backward(phi0, rhs, lam_a, Dx, Dy)
        ctx.grids, ctx.opts = grids, opts
        ctx.lam_scalar, ctx.dx_scalar, ctx.dy_scalar = lam.dim() == 0, D_xx.dim() == 0, D_yy.dim() == 0
        return phi

    @staticmethod
    def backward(ctx, gphi):
        phi0, rhs, lam, Dx, Dy = ctx.saved_tensors
        lib = _lib.load()
        plan = _engine.CACHE.plan(_engine.make_grid(ctx.grids), _engine.make_config(**ctx.opts))
        dev = phi0.device
        ws = _engine.CACHE.workspace(plan, dev)
        abytes = lib.jmg_adjoint_workspace_bytes(plan.handle)
        aws = torch.empty(max(abytes, 1), dtype=torch.uint8, device=dev)
        co = _lib.JmgCoeffs()
        co.lam = lam.data_ptr()
        co.D[0], co.D[1] = Dx.data_ptr(), Dy.data_ptr()
        outs = [torch.empty_like(phi0) for _ in range(5)]
        gphi = gphi.contiguous().to(torch.float64)
        _lib.check(lib.jmg_solve_fixed_vjp(plan.handle, _vp(phi0), _vp(rhs), ctypes.byref(co), _vp(gphi),
                                           *[_vp(o) for o in outs], _vp(ws), ctypes.c_size_t(ws.numel()), _vp(aws),
                                           ctypes.c_size_t(aws.numel()),
                                           ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
        g0, grhs, glam, gdx, gdy = outs
        if ctx.lam_scalar:
            glam = glam.sum()
        if ctx.dx_scalar:
            gdx = gdx.sum()
        if ctx.dy_scalar:
            gdy = gdy.sum()
        return g0, grhs, glam, gdx, gdy, None, None


def solve_2d_fixed_diff(grids, phi0, rhs, lam, D_xx, D_yy, **opts):
    """Differentiable fixed-mode 2D solve on CUDA tensors; returns (phi, count)."""
    if not opts.get("fixed", False):
        raise ValueError("reverse-mode differentiation needs fixed=True, as in the reference")
    dev = next(t.device for t in (phi0, rhs, lam, D_xx, D_yy) if isinstance(t, torch.Tensor))
    def T(x):
        return x if isinstance(x, torch.Tensor) else torch.as_tensor(x, dtype=torch.float64, device=dev)
    phi = FixedSolve2D.apply(T(phi0), T(rhs), T(lam), T(D_xx), T(D_yy), tuple(grids), dict(opts))
    return phi, int(opts.get("max_iters_outer"))
