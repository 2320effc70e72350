"""2D solver front end: ``solve_2d``, its 18 positional wrappers and ``Solver_2D``.

Drop-in for davef96/jsolver's jsolver/solver_2d.py: same names, signatures, defaults,
errors and results. The work runs in libjmg (CUDA, sm_103a) through the C ABI in
include/jmg.h; see ``_engine`` for the argument rules and return types.

Extensions (keyword-only, defaults keep the reference's behaviour):
  stop='distance'|'residual', rtol  -- stop on max|dphi| <= epsilon (reference) or on the
                                       relative residual ||rhs - L_h phi|| / ||rhs|| <= rtol
  precision='fp64'|'mixed'          -- FP32 cycles inside FP64 iterative refinement
  inner_cycles                      -- FP32 cycles per refinement step
  outer='richardson'|'fcg'          -- iterate the cycle as the reference does, or use it
                                       as the preconditioner of flexible CG (needs
                                       stop='residual' or fixed=True)
  guess=None|'learned'|GuessNet     -- start from the learned network's prediction
                                       instead of phi (jsolver_gb300.learned)
"""
import numpy as np

from . import _engine
from ._wrappers import make_wrappers

INT32_MAX = int(np.iinfo(np.int32).max)


def solve_2d(grid_x, grid_y, phi, rhs, lam, D_xx, D_yy, *, D_xy=None, fixed=False, epsilon=1e-12, gamma=1,
             fcycle=False, skip_pre=False, nu1=1, nu2=1, max_iters_outer=INT32_MAX, max_iters_inner=INT32_MAX,
             stop="distance", rtol=1e-10, precision="fp64", inner_cycles=1, guess=None,
             outer="richardson"):
    """Multigrid solve of div(D grad phi) - lam phi = rhs on a padded 2D grid.

    Reference: solve_2d (jsolver/solver_2d.py:196-236). Arrays have shape
    (grid_y.mx + 3, grid_x.mx + 3), float64; ``lam`` and the D components may be
    scalars (all D components scalar, or all arrays). Returns ``(phi, count)``.
    """
    return _engine.solve((grid_x, grid_y), phi, rhs, lam, (D_xx, D_yy), D_xy, fixed=fixed, epsilon=epsilon,
                         gamma=gamma, fcycle=fcycle, skip_pre=skip_pre, nu1=nu1, nu2=nu2,
                         max_iters_outer=max_iters_outer, max_iters_inner=max_iters_inner, stop=stop, rtol=rtol,
                         precision=precision, inner_cycles=inner_cycles, guess=guess, outer=outer)


def solve_2d_batched(grid_x, grid_y, phi, rhs, lam, D_xx, D_yy, *, D_xy=None, lanes=8, fixed=False, epsilon=1e-12,
                     gamma=1, fcycle=False, skip_pre=False, nu1=1, nu2=1, max_iters_outer=INT32_MAX,
                     max_iters_inner=INT32_MAX, stop="distance", rtol=1e-10, precision="fp64", inner_cycles=1,
                     outer="richardson"):
    """B independent 2D solves in one call: jax.vmap(solve_2d) of the reference's
    variational-inference use (README.md:107, examples/benchmark.py:1109-1230).

    ``phi`` and ``rhs`` have shape (B, grid_y.mx + 3, grid_x.mx + 3); each coefficient
    is a scalar, one array shared by the batch, or a (B, ...) array. Returns ``(phi,
    counts)``, counts of length B; problem b's phi and count are solve_2d's on it alone.
    ``lanes`` problems run concurrently (own workspace, stream and graph each)."""
    return _engine.solve_batched((grid_x, grid_y), phi, rhs, lam, (D_xx, D_yy), D_xy, lanes=lanes, fixed=fixed,
                                 epsilon=epsilon, gamma=gamma, fcycle=fcycle, skip_pre=skip_pre, nu1=nu1, nu2=nu2,
                                 max_iters_outer=max_iters_outer, max_iters_inner=max_iters_inner, stop=stop,
                                 rtol=rtol, precision=precision, inner_cycles=inner_cycles, outer=outer)


globals().update(make_wrappers(2, solve_2d))


class Solver_2D:  # noqa: N801 (reference class name)
    """Reference-shaped solver object (jsolver/solver_2d.py:238-692).

    Construction validates the grids (power of 2, coarsest-level efficiency, linear grid)
    with the reference's messages. ``solve`` runs the full GPU solve. After ``setup``
    (or ``solve``), the level operators ``red_black_gauss_seidel``, ``defect``,
    ``prolongate`` and ``distance`` are available on CUDA tensors for inspection.
    """

    def __init__(self, grid_x, grid_y, fixed=False, epsilon=1e-12, gamma=1, fcycle=False, skip_pre=False, nu1=1,
                 nu2=1, max_iters_outer=INT32_MAX, max_iters_inner=INT32_MAX):
        self.grid_x, self.grid_y = grid_x, grid_y
        self.opts = dict(fixed=fixed, epsilon=epsilon, gamma=gamma, fcycle=fcycle, skip_pre=skip_pre, nu1=nu1,
                         nu2=nu2, max_iters_outer=max_iters_outer, max_iters_inner=max_iters_inner)
        self.fixed, self.epsilon, self.gamma, self.fcycle = fixed, epsilon, gamma, fcycle
        self.skip_pre, self.nu1, self.nu2 = skip_pre, nu1, nu2
        self.max_iters_outer, self.max_iters_inner = max_iters_outer, max_iters_inner
        plan = _engine.CACHE.plan(_engine.make_grid((grid_x, grid_y)), _engine.make_config(**self.opts))
        self.levels = plan.levels
        self.mx_level = np.array([grid_x.mx >> l for l in range(self.levels)])
        self.my_level = np.array([grid_y.mx >> l for l in range(self.levels)])
        self.arr_shape = [(int(self.my_level[l]) + 3, int(self.mx_level[l]) + 3) for l in range(self.levels)]
        self.idel_x = grid_x.idel * 0.5 ** np.arange(self.levels)
        self.idel_y = grid_y.idel * 0.5 ** np.arange(self.levels)
        self._ops = None

    def setup(self, lam, D_xx, D_yy, D_xy=None):
        """Builds the coefficient hierarchy on the GPU (compute_discretization, solver_2d.py:385-421)."""
        self._ops = _engine.OperatorSet((self.grid_x, self.grid_y), lam, (D_xx, D_yy), D_xy, **self.opts)
        return self

    def solve(self, phi, rhs, lam, D_xx, D_yy, D_xy=None):
        """solver_2d.py:423-479."""
        return _engine.solve((self.grid_x, self.grid_y), phi, rhs, lam, (D_xx, D_yy), D_xy, **self.opts)

    def _need(self):
        if self._ops is None:
            raise RuntimeError("call setup(lam, D_xx, D_yy) first")
        return self._ops

    def red_black_gauss_seidel(self, phi, rhs, level=0):
        """One RBGS sweep (solver_2d.py:670-692); returns the new phi."""
        return self._need().sweep(phi, rhs, level)

    def defect(self, phi, rhs, level):
        """Defect restricted to level + 1 (solver_2d.py:616-647)."""
        return self._need().restrict(phi, rhs, level)

    def prolongate(self, phi_c, level):
        """Correction interpolated to ``level`` (solver_2d.py:649-668)."""
        ops = self._need()
        z = ops._t(np.zeros(self.arr_shape[level]))
        return ops.prolong_add(z, phi_c, level)

    @staticmethod
    def distance(phi_old, phi):
        """max |phi_old - phi| (solver_2d.py:481-494)."""
        import torch
        if isinstance(phi, torch.Tensor):
            return (phi_old - phi).abs().max()
        return np.max(np.abs(np.asarray(phi_old) - np.asarray(phi)))
