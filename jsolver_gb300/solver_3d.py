"""3D solver front end: ``solve_3d``, its 18 positional wrappers and ``Solver_3D``.

Drop-in for davef96/jsolver's jsolver/solver_3d.py: same names, signatures, defaults,
errors and results; the work runs in libjmg (CUDA, sm_103a) through include/jmg.h.
Keyword extensions as in ``solver_2d`` (stop/rtol, precision, inner_cycles).
"""
import numpy as np

from . import _engine
from ._wrappers import make_wrappers

INT32_MAX = int(np.iinfo(np.int32).max)


def solve_3d(grid_x, grid_y, grid_z, phi, rhs, lam, D_xx, D_yy, D_zz, *, fixed=False, epsilon=1e-12, gamma=1,
             fcycle=False, skip_pre=False, nu1=1, nu2=1, max_iters_outer=INT32_MAX, max_iters_inner=INT32_MAX,
             stop="distance", rtol=1e-10, precision="fp64", inner_cycles=1, outer="richardson"):
    """Multigrid solve on a padded 3D grid (jsolver/solver_3d.py:196-237).

    Arrays have shape (grid_z.mx + 3, grid_y.mx + 3, grid_x.mx + 3), float64. Returns
    ``(phi, count)``.
    """
    return _engine.solve((grid_x, grid_y, grid_z), phi, rhs, lam, (D_xx, D_yy, D_zz), None, fixed=fixed,
                         epsilon=epsilon, gamma=gamma, fcycle=fcycle, skip_pre=skip_pre, nu1=nu1, nu2=nu2,
                         max_iters_outer=max_iters_outer, max_iters_inner=max_iters_inner, stop=stop, rtol=rtol,
                         precision=precision, inner_cycles=inner_cycles, outer=outer)


def solve_3d_batched(grid_x, grid_y, grid_z, phi, rhs, lam, D_xx, D_yy, D_zz, *, lanes=8, fixed=False,
                     epsilon=1e-12, gamma=1, fcycle=False, skip_pre=False, nu1=1, nu2=1, max_iters_outer=INT32_MAX,
                     max_iters_inner=INT32_MAX, stop="distance", rtol=1e-10, precision="fp64", inner_cycles=1,
                     outer="richardson"):
    """B independent 3D solves in one call (jax.vmap(solve_3d)); arguments and results as
    ``solver_2d.solve_2d_batched``, arrays of shape (B, grid_z.mx + 3, grid_y.mx + 3,
    grid_x.mx + 3)."""
    return _engine.solve_batched((grid_x, grid_y, grid_z), phi, rhs, lam, (D_xx, D_yy, D_zz), None, lanes=lanes,
                                 fixed=fixed, epsilon=epsilon, gamma=gamma, fcycle=fcycle, skip_pre=skip_pre,
                                 nu1=nu1, nu2=nu2, max_iters_outer=max_iters_outer, max_iters_inner=max_iters_inner,
                                 stop=stop, rtol=rtol, precision=precision, inner_cycles=inner_cycles, outer=outer)


globals().update(make_wrappers(3, solve_3d))


class Solver_3D:  # noqa: N801 (reference class name)
    """Reference-shaped solver object (jsolver/solver_3d.py:239-706); see ``Solver_2D``."""

    def __init__(self, grid_x, grid_y, grid_z, fixed=False, epsilon=1e-12, gamma=1, fcycle=False, skip_pre=False,
                 nu1=1, nu2=1, max_iters_outer=INT32_MAX, max_iters_inner=INT32_MAX):
        self.grids = (grid_x, grid_y, grid_z)
        self.opts = dict(fixed=fixed, epsilon=epsilon, gamma=gamma, fcycle=fcycle, skip_pre=skip_pre, nu1=nu1,
                         nu2=nu2, max_iters_outer=max_iters_outer, max_iters_inner=max_iters_inner)
        self.fixed, self.epsilon, self.gamma, self.fcycle = fixed, epsilon, gamma, fcycle
        self.skip_pre, self.nu1, self.nu2 = skip_pre, nu1, nu2
        self.max_iters_outer, self.max_iters_inner = max_iters_outer, max_iters_inner
        plan = _engine.CACHE.plan(_engine.make_grid(self.grids), _engine.make_config(**self.opts))
        self.levels = plan.levels
        self.mx_level = np.array([grid_x.mx >> l for l in range(self.levels)])
        self.my_level = np.array([grid_y.mx >> l for l in range(self.levels)])
        self.mz_level = np.array([grid_z.mx >> l for l in range(self.levels)])
        self.arr_shape = [(int(self.mz_level[l]) + 3, int(self.my_level[l]) + 3, int(self.mx_level[l]) + 3)
                          for l in range(self.levels)]
        self.idel_x = grid_x.idel * 0.5 ** np.arange(self.levels)
        self.idel_y = grid_y.idel * 0.5 ** np.arange(self.levels)
        self.idel_z = grid_z.idel * 0.5 ** np.arange(self.levels)
        self._ops = None

    def setup(self, lam, D_xx, D_yy, D_zz):
        """Coefficient hierarchy on the GPU (solver_3d.py:394-429)."""
        self._ops = _engine.OperatorSet(self.grids, lam, (D_xx, D_yy, D_zz), None, **self.opts)
        return self

    def solve(self, phi, rhs, lam, D_xx, D_yy, D_zz):
        """solver_3d.py:431-486."""
        return _engine.solve(self.grids, phi, rhs, lam, (D_xx, D_yy, D_zz), None, **self.opts)

    def _need(self):
        if self._ops is None:
            raise RuntimeError("call setup(lam, D_xx, D_yy, D_zz) first")
        return self._ops

    def red_black_gauss_seidel(self, phi, rhs, level=0):
        return self._need().sweep(phi, rhs, level)

    def defect(self, phi, rhs, level):
        return self._need().restrict(phi, rhs, level)

    def prolongate(self, phi_c, level):
        ops = self._need()
        z = ops._t(np.zeros(self.arr_shape[level]))
        return ops.prolong_add(z, phi_c, level)

    @staticmethod
    def distance(phi_old, phi):
        import torch
        if isinstance(phi, torch.Tensor):
            return (phi_old - phi).abs().max()
        return np.max(np.abs(np.asarray(phi_old) - np.asarray(phi)))
