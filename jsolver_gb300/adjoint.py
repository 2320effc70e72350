"""Differentiation of the solve: reverse mode of the fixed-mode 2D solve (torch.autograd)
and forward mode of every solve (jvp, torch.func.jvp).

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

def _coeffs_struct(lam, D, D_xy):
    """JmgCoeffs over device tensors; 0-d tensors and Python numbers select the scalar form."""
    co = _lib.JmgCoeffs()
    if lam.dim() == 0:
        co.lam, co.lam_scalar = None, float(lam)
    else:
        co.lam = lam.data_ptr()
    for a, d in enumerate(D):
        if d.dim() == 0:
            co.D[a], co.D_scalar[a] = None, float(d)
        else:
            co.D[a] = d.data_ptr()
    co.D_xy = D_xy.data_ptr() if D_xy is not None else None
    return co


def jvp(grids, primals, tangents, **opts):
    """Forward mode of ``solve_2d`` / ``solve_3d``, like ``jax.jvp(solve, primals, tangents)``.

    ``primals`` = (phi0, rhs, lam, D_xx, D_yy[, D_zz][, D_xy]) on one CUDA device (D_xy in
    2D only); ``tangents`` has the same structure, scalar (0-d) where the primal is a
    scalar. Fixed mode and the dynamic distance loop alike: the cycle count follows the
    primal and is not differentiated (jax.jvp through lax.while_loop, solver_2d.py:465-477).
    Returns (phi, phi_dot, count). The tangent is the dual-number solve in libjmg
    (``jmg_solve_jvp``): the solver's own kernels over (value, tangent) pairs, whose value
    part is the plain FP64 solve bit for bit."""
    ndim = len(grids)
    lib = _lib.load()
    dev = next(t.device for t in primals if isinstance(t, torch.Tensor))

    def arr(x):
        return x.detach().to(dev, torch.float64).contiguous() if isinstance(x, torch.Tensor) else \
            torch.as_tensor(x, dtype=torch.float64, device=dev)

    n = 3 + ndim
    if len(primals) not in (n, n + 1) or len(tangents) != len(primals):
        raise ValueError(f"primals and tangents must both be (phi0, rhs, lam, {ndim} D components[, D_xy])")
    P = [arr(x) for x in primals]
    T = [arr(x) for x in tangents]
    phi0, rhs, lam = P[:3]
    D = P[3:n]
    Dxy = P[n] if len(P) > n else None
    t_phi0, t_rhs, t_lam = T[:3]
    t_D = T[3:n]
    t_Dxy = T[n] if len(T) > n else None
    if Dxy is not None and ndim == 3:
        raise ValueError("D_xy is a 2D argument")
    spatial = any(d.dim() > 0 for d in D)
    if spatial:  # the D components are all arrays or all scalars (solver_2d.py:207)
        D = [d.expand(phi0.shape).contiguous() if d.dim() == 0 else d for d in D]
    t_D = [t.expand(d.shape).contiguous() if (t.dim() == 0 and d.dim() > 0) else t for t, d in zip(t_D, D)]
    if t_lam.dim() != lam.dim():
        t_lam = t_lam.expand(lam.shape).contiguous() if lam.dim() else t_lam.sum()
    for d, t in zip(D, t_D):
        if d.dim() != t.dim():
            raise ValueError("tangents of D must be arrays where D is an array, scalars where it is a scalar")
    off = ndim == 2 and spatial and Dxy is not None
    if off and t_Dxy is None:
        t_Dxy = torch.zeros_like(Dxy)
    plan = _engine.CACHE.plan(_engine.make_grid(grids), _engine.make_config(off_diag=off, **opts))
    ws = _engine.CACHE.workspace(plan, dev)
    tws = _engine.CACHE.workspace(plan, dev, "tangent", lib.jmg_tangent_workspace_bytes(plan.handle))
    co = _coeffs_struct(lam, D, Dxy if off else None)
    cd = _coeffs_struct(t_lam, t_D, t_Dxy if off else None)
    phi, phi_dot = torch.empty_like(phi0), torch.empty_like(phi0)
    count = torch.empty((), dtype=torch.int64, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.jmg_solve_jvp(plan.handle, _vp(phi0), _vp(rhs), ctypes.byref(co), _vp(t_phi0), _vp(t_rhs),
                                     ctypes.byref(cd), _vp(phi), _vp(phi_dot), _vp(count), _vp(ws),
                                     ctypes.c_size_t(ws.numel()), _vp(tws), ctypes.c_size_t(tws.numel()),
                                     ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    return phi, phi_dot, count


_dual_solve = jvp  # the name SolveForwardAD.jvp calls


def jvp_2d_fixed(grids, primals, tangents, **opts):
    """Forward mode of the fixed-mode 2D solve (primals and tangents: phi0, rhs, lam, D_xx,
    D_yy); returns (phi, phi_dot)."""
    if not opts.get("fixed", False):
        raise ValueError("jvp_2d_fixed follows the fixed mode: pass fixed=True (jvp() takes both modes)")
    phi, phi_dot, _ = jvp(grids, primals, tangents, **opts)
    return phi, phi_dot


def has_forward_tangent(x):
    """True for a tensor that carries a forward-mode tangent (torch.func.jvp or
    torch.autograd.forward_ad dual tensors)."""
    if not isinstance(x, torch.Tensor):
        return False
    try:
        if torch._C._functorch.is_functorch_wrapped_tensor(x):
            return True
    except AttributeError:  # pragma: no cover
        pass
    return torch.autograd.forward_ad.unpack_dual(x).tangent is not None


def _outside_functorch():
    """Runs the library call with torch.func's interpreter stack cleared, so that tensors
    created for it (copies, outputs, workspaces) are plain tensors with storage."""
    try:
        from torch._functorch.pyfunctorch import temporarily_clear_interpreter_stack
        return temporarily_clear_interpreter_stack()
    except ImportError:  # pragma: no cover
        import contextlib
        return contextlib.nullcontext()


def _storage_tensor(x):
    """The plain tensor under torch.func's wrappers, live or dead (the level of a saved
    tensor may have exited by the time the forward-mode rule runs); the library reads
    device pointers."""
    f = torch._C._functorch
    for _ in range(64):
        if hasattr(f, "unwrap_if_dead"):
            x = f.unwrap_if_dead(x)
        if f.is_functorch_wrapped_tensor(x) or f.is_gradtrackingtensor(x):
            x = f.get_unwrapped(x)
            continue
        break
    return x


class SolveForwardAD(torch.autograd.Function):
    """solve_2d / solve_3d as a torch function with a forward-mode rule: under
    ``torch.func.jvp`` or ``torch.autograd.forward_ad`` the tangent of phi comes from the
    dual-number solve (``jmg_solve_jvp``); the count is not differentiable."""

    @staticmethod
    def forward(grids, opts, has_dxy, *xs):
        xs = [_storage_tensor(torch.autograd.forward_ad.unpack_dual(x).primal) if isinstance(x, torch.Tensor) else x
              for x in xs]
        ndim = len(grids)
        with _outside_functorch():
            phi, count = _engine.solve(grids, xs[0], xs[1], xs[2], tuple(xs[3:3 + ndim]),
                                       xs[3 + ndim] if has_dxy else None, **opts)
        if not isinstance(count, torch.Tensor):
            count = torch.tensor(count, dtype=torch.int64, device=phi.device)
        return phi, count

    @staticmethod
    def setup_context(ctx, inputs, output):
        grids, opts, has_dxy = inputs[:3]
        ctx.grids, ctx.opts, ctx.has_dxy = grids, opts, has_dxy
        xs = inputs[3:]
        ctx.kinds = [isinstance(x, torch.Tensor) for x in xs]
        ctx.scalars = [None if isinstance(x, torch.Tensor) else float(x) for x in xs]
        # the primals' storage, taken while their torch.func levels are alive (the rule
        # below reads device pointers only)
        ctx.storage = [_storage_tensor(x) for x in xs if isinstance(x, torch.Tensor)]
        ctx.mark_non_differentiable(output[1])

    @staticmethod
    def jvp(ctx, g_grids, g_opts, g_has_dxy, *gxs):
        saved = list(ctx.storage)
        primals, tangents = [], []
        dev = saved[0].device
        for kind, sc, g in zip(ctx.kinds, ctx.scalars, gxs):
            if kind:
                x = saved.pop(0)
                primals.append(x)
                tangents.append(_storage_tensor(g) if g is not None else torch.zeros_like(x))
            else:
                primals.append(torch.tensor(sc, dtype=torch.float64, device=dev))
                tangents.append(torch.zeros((), dtype=torch.float64, device=dev))
        with _outside_functorch():
            _, phi_dot, _ = _dual_solve(ctx.grids, primals, tangents, **ctx.opts)
        return phi_dot, None


def solve_forward_ad(grids, phi, rhs, lam, D, D_xy, **opts):
    """The solve through SolveForwardAD (CUDA tensors carrying forward-mode tangents)."""
    xs = [phi, rhs, lam] + list(D) + ([D_xy] if D_xy is not None else [])
    phi_out, count = SolveForwardAD.apply(tuple(grids), dict(opts), D_xy is not None, *xs)
    if opts.get("fixed", False):
        return phi_out, int(opts.get("max_iters_outer"))
    return phi_out, count
