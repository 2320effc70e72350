"""Host side of a solve: argument rules of the reference, plan/workspace caching, C-ABI calls.

``solve`` mirrors ``Solver_2D.solve`` / ``Solver_3D.solve`` (jsolver/solver_2d.py:423-479,
jsolver/solver_3d.py:431-486): the same validation order and messages (grid checks when
the solver is constructed, then dtype, then shapes), the same scalar/array forms of
``lam`` and ``D``, the same return value ``(phi, count)``.

Return types follow the inputs: NumPy/Python inputs give a NumPy ``phi`` and a Python
``int`` count (the call waits for the GPU, like ``block_until_ready``); CUDA-tensor inputs
give a CUDA tensor and, in dynamic mode, a 0-d int64 CUDA tensor count without any host
synchronisation (fixed mode returns ``max_iters_outer`` as an int, as the reference does).
"""
import ctypes
import threading

import numpy as np
import torch

from . import _lib
from ._arrays import (is_cuda_tensor, is_float64, is_scalar, pick_device, scalar_value, shape_of,
                      to_device)

INT32_MAX = int(np.iinfo(np.int32).max)

_PREC = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}
_STOP = {"distance": _lib.STOP_DISTANCE, "residual": _lib.STOP_RESIDUAL}
_OUTER = {"richardson": _lib.OUTER_RICHARDSON, "fcg": _lib.OUTER_FCG}


def make_config(fixed=False, epsilon=1e-12, gamma=1, fcycle=False, skip_pre=False, nu1=1, nu2=1,
                max_iters_outer=INT32_MAX, max_iters_inner=INT32_MAX, stop="distance", rtol=1e-10,
                precision="fp64", inner_cycles=1, outer="richardson", off_diag=False):
    c = _lib.default_config()
    c.fixed = int(bool(fixed))
    c.epsilon = float(epsilon)
    c.gamma = int(gamma)
    c.fcycle = int(bool(fcycle))
    c.skip_pre = int(bool(skip_pre))
    c.nu1 = int(nu1)
    c.nu2 = int(nu2)
    c.max_iters_outer = int(max_iters_outer)
    c.max_iters_inner = int(max_iters_inner)
    if stop not in _STOP:
        raise ValueError(f"stop must be one of {sorted(_STOP)}, got {stop!r}")
    if precision not in _PREC:
        raise ValueError(f"precision must be one of {sorted(_PREC)}, got {precision!r}")
    c.stop = _STOP[stop]
    c.rtol = float(rtol)
    c.precision = _PREC[precision]
    c.inner_cycles = int(inner_cycles)
    if outer not in _OUTER:
        raise ValueError(f"outer must be one of {sorted(_OUTER)}, got {outer!r}")
    c.outer = _OUTER[outer]
    c.off_diag = int(bool(off_diag))
    return c


def make_grid(grids):
    g = _lib.JmgGrid()
    g.ndim = len(grids)
    for a, gr in enumerate(grids):
        g.m[a] = int(gr.mx)
        g.idel[a] = float(gr.idel)
        g.is_linear[a] = int(bool(gr.is_linear))
    return g


def _cfg_key(c):
    return tuple(getattr(c, f) for f, _ in c._fields_)


def _grid_key(g):
    return (g.ndim, tuple(g.m), tuple(g.idel), tuple(g.is_linear))


class _Cache:
    """Plans (with their captured graphs) and workspaces, reused across calls."""

    def __init__(self):
        self.lock = threading.Lock()
        self.plans = {}
        self.ws = {}

    def plan(self, grid, cfg):
        key = (_grid_key(grid), _cfg_key(cfg))
        with self.lock:
            p = self.plans.get(key)
            if p is None:
                p = _lib.Plan(grid, cfg)
                self.plans[key] = p
            return p

    def workspace(self, plan, device, kind="solve", nbytes=None):
        """Device workspace of a plan, kept across calls (a stable address lets the
        library reuse the graphs it captured for that address)."""
        nbytes = plan.workspace_bytes if nbytes is None else nbytes
        key = (id(plan), str(device), kind)
        with self.lock:
            w = self.ws.get(key)
            if w is None or w.numel() < nbytes:
                w = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=device)
                self.ws[key] = w
            return w


CACHE = _Cache()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream_ptr(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def validate(ndim, phi, rhs, lam, D, D_xy, expected_shape):
    """dtype and shape rules of solver_2d.py:444-453 / solver_3d.py:452-460."""
    args = [phi, rhs, lam] + list(D) + ([] if D_xy is None else [D_xy])
    if not all(is_float64(a) for a in args):
        raise ValueError("Incorrect configuration: dtype must be 'jnp.float64' for all arguments.")
    s = shape_of
    sl = is_scalar(lam)
    spatial = not all(is_scalar(d) for d in D)
    off = ndim == 2 and spatial and D_xy is not None
    same_D = all(s(d) == s(D[0]) for d in D)
    bad = (not same_D or (sl and not s(phi) == s(rhs)) or (not sl and not s(phi) == s(rhs) == s(lam))
           or (spatial and not all(s(phi) == s(x) for x in [rhs] + list(D)))
           or (off and not s(phi) == s(D_xy)) or s(phi) != tuple(expected_shape))
    if bad:
        names = ["D_xx", "D_yy", "D_zz"][:ndim]
        dstr = ", ".join(f"{n}={s(d)}" for n, d in zip(names, D))
        tail = f", D_xy={'None' if D_xy is None else s(D_xy)}" if ndim == 2 else ""
        raise ValueError(f"Shape mismatch: phi={s(phi)}, rhs={s(rhs)}, lam={s(lam)}, {dstr}{tail}.")
    return sl, spatial, off


def expected_shape(grids):
    return tuple(int(g.mx) + 3 for g in reversed(grids))


class Prepared:
    """Device-side arguments of one call (keeps the tensors alive)."""

    def __init__(self, ndim, device, lam, D, D_xy, sl, spatial):
        self.coeffs = _lib.JmgCoeffs()
        self.keep = []
        if sl:
            self.coeffs.lam = None
            self.coeffs.lam_scalar = scalar_value(lam)
        else:
            t = to_device(lam, device)
            self.keep.append(t)
            self.coeffs.lam = t.data_ptr()
        for a in range(ndim):
            if spatial:
                t = to_device(D[a], device)
                self.keep.append(t)
                self.coeffs.D[a] = t.data_ptr()
            else:
                self.coeffs.D[a] = None
                self.coeffs.D_scalar[a] = scalar_value(D[a])
        self.coeffs.D_xy = None
        if D_xy is not None and spatial:
            t = to_device(D_xy, device)
            self.keep.append(t)
            self.coeffs.D_xy = t.data_ptr()


def solve(grids, phi, rhs, lam, D, D_xy=None, guess=None, **opts):
    """Full solve through ``jmg_solve``. ``grids`` is (grid_x, grid_y[, grid_z]).

    ``guess``: None starts from ``phi`` (the reference); ``"learned"`` (the package's
    trained network) or a ``learned.GuessNet`` replaces phi's values by the network's
    prediction (2D square grids; phi still fixes the shape and dtype rules)."""
    ndim = len(grids)
    grid = make_grid(grids)
    CACHE.plan(grid, make_config(**opts))  # grid checks first (Solver_2D.__init__)
    sl, spatial, off = validate(ndim, phi, rhs, lam, D, D_xy, expected_shape(grids))
    cfg = make_config(off_diag=off, **opts)
    plan = CACHE.plan(grid, cfg)
    torch_in = any(is_cuda_tensor(a) for a in [phi, rhs, lam] + list(D))
    args = [phi, rhs, lam] + list(D) + ([] if D_xy is None else [D_xy])
    from .adjoint import has_forward_tangent
    if any(has_forward_tangent(a) for a in args):
        # forward mode (torch.func.jvp / forward_ad): jax.jvp of the reference's solve
        if guess is not None:
            raise ValueError("guess= is available for 2D solves without gradients")
        if cfg.precision != _lib.PREC_FP64 or cfg.outer != _lib.OUTER_RICHARDSON or \
                (not cfg.fixed and cfg.stop != _lib.STOP_DISTANCE):
            raise NotImplementedError("forward mode differentiates the reference's FP64 iteration (fixed count or "
                                      "the distance stop)")
        from .adjoint import solve_forward_ad
        return solve_forward_ad(grids, phi, rhs, lam, D, D_xy, **opts)
    wants_grad = torch.is_grad_enabled() and any(isinstance(a, torch.Tensor) and a.requires_grad for a in args)
    if guess is not None and (ndim != 2 or wants_grad):
        raise ValueError("guess= is available for 2D solves without gradients")
    if wants_grad:
        if not cfg.fixed:
            raise ValueError("reverse-mode differentiation needs fixed=True, as in the reference "
                             "(its dynamic while_loop is not reverse-differentiable)")
        if cfg.precision != _lib.PREC_FP64 or cfg.outer != _lib.OUTER_RICHARDSON:
            raise NotImplementedError("the hand-written adjoint differentiates the reference's FP64 fixed-mode "
                                      "iteration (precision fp64, outer richardson)")
        from .adjoint import solve_fixed_diff
        return solve_fixed_diff(grids, phi, rhs, lam, D, D_xy if off else None, **opts)
    device = pick_device(phi, rhs, lam, *D)
    _lib.load()
    with torch.cuda.device(device):
        phi_d = to_device(phi, device)
        rhs_d = to_device(rhs, device)
        if guess is not None:
            from .learned import predict_phi0
            phi_d = predict_phi0(guess, grids, rhs_d, lam, D, device)
        prep = Prepared(ndim, device, lam, D, D_xy, sl, spatial)
        out = torch.empty_like(phi_d)
        count = torch.empty((), dtype=torch.int64, device=device)
        ws = CACHE.workspace(plan, device)
        _lib.check(_lib.load().jmg_solve(plan.handle, _ptr(phi_d), _ptr(rhs_d), ctypes.byref(prep.coeffs),
                                         _ptr(out), _ptr(count), _ptr(ws), ctypes.c_size_t(ws.numel()),
                                         _stream_ptr(device)))
        if torch_in:
            return out, (int(cfg.max_iters_outer) if cfg.fixed else count)
        # host inputs wait for the result anyway: confirm that no device-side wait ran out
        _lib.check(_lib.load().jmg_solve_check(plan.handle, _ptr(ws), ctypes.c_size_t(ws.numel()),
                                               _stream_ptr(device)))
        return out.cpu().numpy(), (int(cfg.max_iters_outer) if cfg.fixed else int(count.item()))


def solve_batched(grids, phi, rhs, lam, D, D_xy=None, lanes=8, **opts):
    """B independent solves of one grid through ``jmg_solve_batched``.

    ``phi`` and ``rhs`` have shape (B, *spatial); ``lam`` and every D component are a
    scalar, one array of the spatial shape shared by all problems, or a (B, *spatial)
    array (the reference's jax.vmap over solve_2d / solve_3d with those in_axes). ``lanes``
    problems run side by side, each on its own workspace and stream. Returns ``(phi,
    counts)`` with counts an int64 array of length B; problem b's results are those of
    ``solve`` on problem b alone."""
    ndim = len(grids)
    grid = make_grid(grids)
    CACHE.plan(grid, make_config(**opts))  # grid checks first
    spatial_shape = expected_shape(grids)
    ps, rs = shape_of(phi), shape_of(rhs)
    if len(ps) != ndim + 1 or ps != rs or ps[0] < 1:
        raise ValueError(f"Shape mismatch: batched phi and rhs must both have shape (B, "
                         f"{', '.join(map(str, spatial_shape))}) with B >= 1, got phi={ps}, rhs={rs}.")
    nb = ps[0]
    coeffs = [lam] + list(D) + ([] if D_xy is None else [D_xy])

    def batched(x):
        return not is_scalar(x) and len(shape_of(x)) == ndim + 1

    for x in coeffs:
        if batched(x) and shape_of(x)[0] != nb:
            raise ValueError(f"Shape mismatch: batched coefficient of shape {shape_of(x)} for a batch of {nb}.")

    def first(x):  # problem 0's view
        return x[0] if batched(x) else x

    sl, spatial, off = validate(ndim, phi[0], rhs[0], first(lam), [first(d) for d in D],
                                None if D_xy is None else first(D_xy), spatial_shape)
    cfg = make_config(off_diag=off, **opts)
    plan = CACHE.plan(grid, cfg)
    torch_in = any(is_cuda_tensor(a) for a in [phi, rhs] + coeffs)
    device = pick_device(phi, rhs, *coeffs)
    lib = _lib.load()
    npts = int(np.prod(spatial_shape))
    with torch.cuda.device(device):
        phi_d = to_device(phi, device)
        rhs_d = to_device(rhs, device)
        prep = Prepared(ndim, device, lam, D, D_xy, sl, spatial)
        st = _lib.JmgBatchStrides()
        st.lam = npts if (not sl and batched(lam)) else 0
        for a in range(ndim):
            st.D[a] = npts if (spatial and batched(D[a])) else 0
        st.D_xy = npts if (off and batched(D_xy)) else 0
        out = torch.empty_like(phi_d)
        counts = torch.empty(nb, dtype=torch.int64, device=device)
        lanes = max(1, min(int(lanes), nb, 32))
        ws = CACHE.workspace(plan, device, "batch", lib.jmg_batched_workspace_bytes(plan.handle, lanes))
        _lib.check(lib.jmg_solve_batched(plan.handle, nb, _ptr(phi_d), _ptr(rhs_d), ctypes.byref(prep.coeffs),
                                         ctypes.byref(st), _ptr(out), _ptr(counts), _ptr(ws),
                                         ctypes.c_size_t(ws.numel()), _stream_ptr(device)))
        if torch_in:
            return out, counts
        return out.cpu().numpy(), counts.cpu().numpy()


class OperatorSet:
    """Level operators of one problem (reference Solver methods) on CUDA tensors."""

    def __init__(self, grids, lam, D, D_xy=None, **opts):
        self.ndim = len(grids)
        self.grids = grids
        sl, spatial, off = validate(self.ndim, np.zeros(expected_shape(grids)), np.zeros(expected_shape(grids)),
                                    lam, D, D_xy, expected_shape(grids))
        self.cfg = make_config(off_diag=off, **opts)
        self.plan = _lib.Plan(make_grid(grids), self.cfg)
        self.device = pick_device(lam, *D)
        self.prep = Prepared(self.ndim, self.device, lam, D, D_xy, sl, spatial)
        self.ws = torch.empty(max(self.plan.workspace_bytes, 1), dtype=torch.uint8, device=self.device)
        self.lib = _lib.load()
        _lib.check(self.lib.jmg_build_hierarchy(self.plan.handle, ctypes.byref(self.prep.coeffs), _ptr(self.ws),
                                                ctypes.c_size_t(self.ws.numel()), _stream_ptr(self.device)))
        ms = [int(g.mx) for g in grids]
        self.shapes = [tuple((m >> l) + 3 for m in reversed(ms)) for l in range(self.plan.levels)]

    def _t(self, x):
        return to_device(x, self.device).clone()

    def _args(self):
        return _ptr(self.ws), ctypes.c_size_t(self.ws.numel()), _stream_ptr(self.device)

    def sweep(self, phi, rhs, level=0):
        p = self._t(phi)
        r = self._t(rhs)
        _lib.check(self.lib.jmg_op_sweep(self.plan.handle, level, _ptr(p), _ptr(r), *self._args()))
        return p

    def restrict(self, phi, rhs, level):
        p, r = self._t(phi), self._t(rhs)
        out = torch.zeros(self.shapes[level + 1], dtype=torch.float64, device=self.device)
        _lib.check(self.lib.jmg_op_restrict(self.plan.handle, level, _ptr(p), _ptr(r), _ptr(out), *self._args()))
        return out

    def prolong_add(self, phi, phi_c, level):
        p, c = self._t(phi), self._t(phi_c)
        _lib.check(self.lib.jmg_op_prolong(self.plan.handle, level, _ptr(p), _ptr(c), *self._args()))
        return p

    def residual(self, phi, rhs, level=0):
        p, r = self._t(phi), self._t(rhs)
        out = torch.empty(self.shapes[level], dtype=torch.float64, device=self.device)
        _lib.check(self.lib.jmg_op_residual(self.plan.handle, level, _ptr(p), _ptr(r), _ptr(out), *self._args()))
        return out

    def coeff(self, level, which):
        out = torch.empty(self.shapes[level], dtype=torch.float64, device=self.device)
        _lib.check(self.lib.jmg_op_coeff(self.plan.handle, level, which, _ptr(out), *self._args()))
        return out

    def rel_residual(self, phi, rhs):
        p, r = self._t(phi), self._t(rhs)
        out = torch.empty((), dtype=torch.float64, device=self.device)
        _lib.check(self.lib.jmg_rel_residual(self.plan.handle, _ptr(p), _ptr(r), _ptr(out), *self._args()))
        return out
