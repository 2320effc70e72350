"""Differentiation of the solve: reverse mode of the fixed-mode solve (torch.autograd) and
forward mode of every solve (jvp, torch.func.jvp).

The reference differentiates ``solve_2d(..., fixed=True)`` and ``solve_3d(..., fixed=True)``
with ``jax.vjp`` (jsolver/solver_2d.py:18-26, solver_3d.py:468-470; README: reverse mode
works in fixed mode only). Here the vector-Jacobian product is the hand-written adjoint in
libjmg (``jmg_solve_fixed_vjp_nd``: transposed smoother, restriction and prolongation
swapped, per-cycle checkpointing with recomputation, backward of the coefficient
hierarchy), for 2D and 3D and the 5-, 7- and 9-point (D_xy) stencils. ``solve_2d`` and
``solve_3d`` route CUDA tensors that require grad through ``FixedSolve`` when
``fixed=True``.
"""
import ctypes

import torch

from . import _engine, _lib


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _full(x, shape):
    return x.expand(shape).contiguous() if x.dim() == 0 else x.contiguous()


class FixedSolve(torch.autograd.Function):
    """phi_n = solve(grids, phi0, rhs, lam, D[, D_xy], fixed=True, ...) with
    xs = (phi0, rhs, lam, D_xx, D_yy[, D_zz][, D_xy])."""

    @staticmethod
    def forward(ctx, grids, opts, has_dxy, *xs):
        ndim = len(grids)
        shape = xs[0].shape
        phi0, rhs = xs[0].contiguous(), xs[1].contiguous()
        lam = _full(xs[2], shape)
        D = tuple(_full(d, shape) for d in xs[3:3 + ndim])
        Dxy = xs[3 + ndim].contiguous() if has_dxy else None
        with torch.no_grad():
            phi, _ = _engine.solve(grids, phi0, rhs, lam, D, Dxy, **opts)
        ctx.save_for_backward(phi0, rhs, lam, *D, *([Dxy] if has_dxy else []))
        ctx.grids, ctx.opts, ctx.has_dxy = grids, opts, has_dxy
        ctx.scalar = [x.dim() == 0 for x in xs]
        return phi

    @staticmethod
    def backward(ctx, gphi):
        saved = ctx.saved_tensors
        ndim = len(ctx.grids)
        phi0, rhs, lam = saved[:3]
        D = saved[3:3 + ndim]
        lib = _lib.load()
        cfg = _engine.make_config(off_diag=ctx.has_dxy, **ctx.opts)
        plan = _engine.CACHE.plan(_engine.make_grid(ctx.grids), cfg)
        dev = phi0.device
        ws = _engine.CACHE.workspace(plan, dev)
        abytes = lib.jmg_adjoint_workspace_bytes(plan.handle)
        aws = _engine.CACHE.workspace(plan, dev, "adjoint", abytes)
        co = _lib.JmgCoeffs()
        co.lam = lam.data_ptr()
        for a, d in enumerate(D):
            co.D[a] = d.data_ptr()
        co.D_xy = saved[3 + ndim].data_ptr() if ctx.has_dxy else None
        outs = [torch.empty_like(phi0) for _ in range(3 + ndim + (1 if ctx.has_dxy else 0))]
        dbar = (ctypes.c_void_p * 3)(*[o.data_ptr() for o in outs[3:3 + ndim]])
        gphi = gphi.contiguous().to(torch.float64)
        _lib.check(lib.jmg_solve_fixed_vjp_nd(
            plan.handle, _vp(phi0), _vp(rhs), ctypes.byref(co), _vp(gphi), _vp(outs[0]), _vp(outs[1]),
            _vp(outs[2]), dbar, _vp(outs[3 + ndim]) if ctx.has_dxy else None, _vp(ws), ctypes.c_size_t(ws.numel()),
            _vp(aws), ctypes.c_size_t(aws.numel()), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
        # a scalar input's gradient is the sum over the array it stood for
        grads = [o.sum() if sc else o for o, sc in zip(outs, ctx.scalar)]
        return (None, None, None, *grads)


def solve_fixed_diff(grids, phi0, rhs, lam, D, D_xy=None, **opts):
    """Differentiable fixed-mode solve (2D or 3D, optional D_xy) on CUDA tensors; returns
    (phi, count)."""
    if not opts.get("fixed", False):
        raise ValueError("reverse-mode differentiation needs fixed=True, as in the reference")
    args = [phi0, rhs, lam, *D] + ([D_xy] if D_xy is not None else [])
    dev = next(t.device for t in args if isinstance(t, torch.Tensor))

    def T(x):
        return x if isinstance(x, torch.Tensor) else torch.as_tensor(x, dtype=torch.float64, device=dev)

    phi = FixedSolve.apply(tuple(grids), dict(opts), D_xy is not None, *[T(a) for a in args])
    return phi, int(opts.get("max_iters_outer"))


def solve_2d_fixed_diff(grids, phi0, rhs, lam, D_xx, D_yy, **opts):
    """The 2D 5-point form of ``solve_fixed_diff``."""
    return solve_fixed_diff(grids, phi0, rhs, lam, (D_xx, D_yy), **opts)


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
