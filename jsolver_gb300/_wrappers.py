"""Generates the reference's positional wrapper functions for solve_2d / solve_3d.

The reference defines 18 wrappers per dimension (jsolver/solver_2d.py:10-194,
jsolver/solver_3d.py:10-194): {dynamic, fixed(iters_outer, iters_inner),
fixed_simple(iters; iters_inner = 1)} x {V, F, W} x {normal, skip_pre}.
Their names, positional signatures and keyword settings are reproduced here.
"""

# (name suffix, extra keyword settings) in the reference's order
CYCLES = [
    ("", {}),
    ("_skip_pre", {"skip_pre": True}),
    ("_fcycle", {"fcycle": True}),
    ("_fcycle_skip_pre", {"fcycle": True, "skip_pre": True}),
    ("_wcycle", {"gamma": 2}),
    ("_wcycle_skip_pre", {"gamma": 2, "skip_pre": True}),
]


def make_wrappers(ndim, solve):
    """Return {name: function} for the 18 wrappers of ``solve_{ndim}d``."""
    pre = f"solve_{ndim}d"
    out = {}
    for suffix, kw in CYCLES:
        kw = dict(kw)
        if ndim == 2:
            def simple(grid_x, grid_y, phi, rhs, lam, D_xx, D_yy, D_xy=None, _kw=kw):
                return solve(grid_x=grid_x, grid_y=grid_y, phi=phi, rhs=rhs, lam=lam, D_xx=D_xx, D_yy=D_yy,
                             D_xy=D_xy, **_kw)

            def fixed(grid_x, grid_y, iters_outer, iters_inner, phi, rhs, lam, D_xx, D_yy, D_xy=None, _kw=kw):
                return solve(grid_x=grid_x, grid_y=grid_y, fixed=True, max_iters_outer=iters_outer,
                             max_iters_inner=iters_inner, phi=phi, rhs=rhs, lam=lam, D_xx=D_xx, D_yy=D_yy,
                             D_xy=D_xy, **_kw)

            def fixed_simple(grid_x, grid_y, iters, phi, rhs, lam, D_xx, D_yy, D_xy=None, _fixed=fixed):
                return _fixed(grid_x, grid_y, iters, 1, phi, rhs, lam, D_xx, D_yy, D_xy)
        else:
            def simple(grid_x, grid_y, grid_z, phi, rhs, lam, D_xx, D_yy, D_zz, _kw=kw):
                return solve(grid_x=grid_x, grid_y=grid_y, grid_z=grid_z, phi=phi, rhs=rhs, lam=lam, D_xx=D_xx,
                             D_yy=D_yy, D_zz=D_zz, **_kw)

            def fixed(grid_x, grid_y, grid_z, iters_outer, iters_inner, phi, rhs, lam, D_xx, D_yy, D_zz, _kw=kw):
                return solve(grid_x=grid_x, grid_y=grid_y, grid_z=grid_z, fixed=True, max_iters_outer=iters_outer,
                             max_iters_inner=iters_inner, phi=phi, rhs=rhs, lam=lam, D_xx=D_xx, D_yy=D_yy,
                             D_zz=D_zz, **_kw)

            def fixed_simple(grid_x, grid_y, grid_z, iters, phi, rhs, lam, D_xx, D_yy, D_zz, _fixed=fixed):
                return _fixed(grid_x, grid_y, grid_z, iters, 1, phi, rhs, lam, D_xx, D_yy, D_zz)
        base = suffix
        names = {
            f"{pre}{base}_simple": simple,
            f"{pre}_fixed{base}_simple": fixed_simple,
            f"{pre}_fixed{base}": fixed,
        }
        for n, f in names.items():
            f.__name__ = n
            f.__qualname__ = n
            f.__doc__ = (f"Positional wrapper of ``{pre}`` with settings {kw or 'default (V-cycle)'}"
                         f"{'; fixed number of cycles' if 'fixed' in n else ''}"
                         f"{' (iters_inner = 1)' if n.endswith('_simple') and 'fixed' in n else ''}.")
            out[n] = f
    return out
