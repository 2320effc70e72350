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
        aws = _engine.CACHE.workspace(plan, dev, "adjoint", abytes)
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


# ---- forward mode ----------------------------------------------------------------------

def jvp_2d_fixed(grids, primals, tangents, **opts):
    """Forward mode of the fixed-mode 2D solve, like ``jax.jvp(solve, primals, tangents)``.

    ``primals`` and ``tangents`` are (phi0, rhs, lam, D_xx, D_yy) on one CUDA device;
    scalar lam / D take scalar tangents. Returns (phi, phi_dot). The tangent is the
    dual-number solve in libjmg (``jmg_solve_fixed_jvp``): the coefficient hierarchy of
    the tangent coefficients (linear, with d(1/A_cc) = -(1/A_cc)^2 dA_cc) and the
    reference's schedule with dual sweeps and restrictions.
    """
    if not opts.get("fixed", False):
        raise ValueError("the tangent follows the fixed mode: pass fixed=True")
    lib = _lib.load()
    dev = next(t.device for t in primals if isinstance(t, torch.Tensor))

    def arr(x):
        return x.to(dev, torch.float64).contiguous() if isinstance(x, torch.Tensor) else \
            torch.as_tensor(x, dtype=torch.float64, device=dev)

    phi0, rhs, lam, Dx, Dy = [arr(x) for x in primals]
    t_phi0, t_rhs, t_lam, t_Dx, t_Dy = [arr(x) for x in tangents]
    plan = _engine.CACHE.plan(_engine.make_grid(grids), _engine.make_config(**opts))
    ws = _engine.CACHE.workspace(plan, dev)
    tws = torch.empty(max(lib.jmg_tangent_workspace_bytes(plan.handle), 1), dtype=torch.uint8, device=dev)

    def coeffs(lm, dx, dy):
        co = _lib.JmgCoeffs()
        if lm.dim() == 0:
            co.lam, co.lam_scalar = None, float(lm)
        else:
            co.lam = lm.data_ptr()
        for a, d in enumerate((dx, dy)):
            if d.dim() == 0:
                co.D[a], co.D_scalar[a] = None, float(d)
            else:
                co.D[a] = d.data_ptr()
        return co

    if (Dx.dim() == 0) != (Dy.dim() == 0):
        Dx, Dy = Dx.expand(phi0.shape).contiguous(), Dy.expand(phi0.shape).contiguous()
        t_Dx, t_Dy = t_Dx.expand(phi0.shape).contiguous(), t_Dy.expand(phi0.shape).contiguous()
    if t_lam.dim() != lam.dim():
        t_lam = t_lam.expand(lam.shape).contiguous() if lam.dim() else t_lam.sum()
    for a in range(2):
        pa, ta = (Dx, Dy)[a], (t_Dx, t_Dy)[a]
        if ta.dim() != pa.dim():
            raise ValueError("tangents of D must be arrays where D is an array, scalars where it is a scalar")
    co, cd = coeffs(lam, Dx, Dy), coeffs(t_lam, t_Dx, t_Dy)
    phi, phi_dot = torch.empty_like(phi0), torch.empty_like(phi0)
    _lib.check(lib.jmg_solve_fixed_jvp(plan.handle, _vp(phi0), _vp(rhs), ctypes.byref(co), _vp(t_phi0), _vp(t_rhs),
                                       ctypes.byref(cd), _vp(phi), _vp(phi_dot), _vp(ws), ctypes.c_size_t(ws.numel()),
                                       _vp(tws), ctypes.c_size_t(tws.numel()),
                                       ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    return phi, phi_dot
