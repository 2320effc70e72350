"""The solve as PyTorch operators: ``torch.ops.jmg.solve_2d`` and ``torch.ops.jmg.solve_3d``.

``torch.library`` custom operators over the same C ABI call as ``solver_2d.solve_2d`` /
``solver_3d.solve_3d`` (jsolver/solver_2d.py:196-236, solver_3d.py:196-237), so that
torch code can put the solve into graphs that ``torch.compile`` or ``torch.export``
trace: each has a fake (shape-only) implementation for tracing and runs the CUDA solve on
the inputs' device and current stream (host tensors are solved on the current GPU and
returned on the host). Grids are passed as per-axis (m, xb, xe, centered) lists;
coefficients as tensors, 0-d for a scalar. The operators return ``(phi, count)`` with
``count`` a 0-d int64 tensor on the inputs' device. Reverse-mode differentiation is
not registered here: it goes through ``solve_2d(..., fixed=True)`` (jsolver_gb300.adjoint).

Example::

    from jsolver_gb300 import torch_ops  # registers the operators
    phi, count = torch.ops.jmg.solve_2d(phi0, rhs, lam, Dxx, Dyy, None, [m, m], [0.0, 0.0],
                                         [1.0, 1.0], [True, True], *torch_ops.options())
"""
from typing import List, Optional, Tuple

import torch

from . import _engine
from .grid_1d import grid_1D

INT32_MAX = 2147483647
_OPTION_NAMES = ("fixed", "epsilon", "gamma", "fcycle", "skip_pre", "nu1", "nu2", "max_iters_outer", "stop", "rtol",
                 "precision", "inner_cycles", "outer")


def options(fixed=False, epsilon=1e-12, gamma=1, fcycle=False, skip_pre=False, nu1=1, nu2=1,
            max_iters_outer=INT32_MAX, stop="distance", rtol=1e-10, precision="fp64", inner_cycles=1,
            outer="richardson"):
    """The solver options in the operators' positional order, with solve_2d's defaults."""
    return (bool(fixed), float(epsilon), int(gamma), bool(fcycle), bool(skip_pre), int(nu1), int(nu2),
            int(max_iters_outer), str(stop), float(rtol), str(precision), int(inner_cycles), str(outer))


def _grids(m, xb, xe, centered):
    return tuple(grid_1D(int(m[a]), float(xb[a]), float(xe[a]), centered=bool(centered[a])) for a in range(len(m)))


def _run(grids, phi0, rhs, lam, D, D_xy, opts):
    kw = dict(zip(_OPTION_NAMES, opts))
    phi, count = _engine.solve(grids, phi0, rhs, lam, D, D_xy, **kw)
    # host tensors are solved on the GPU and come back as NumPy: return them as tensors
    # on phi0's device, like the inputs
    if not isinstance(phi, torch.Tensor):
        phi = torch.from_numpy(phi).to(phi0.device)
    if not isinstance(count, torch.Tensor):
        count = torch.tensor(count, dtype=torch.int64, device=phi0.device)
    return phi, count.to(phi0.device).reshape(())


@torch.library.custom_op("jmg::solve_2d", mutates_args=())
def solve_2d(phi0: torch.Tensor, rhs: torch.Tensor, lam: torch.Tensor, D_xx: torch.Tensor, D_yy: torch.Tensor,
             D_xy: Optional[torch.Tensor], m: List[int], xb: List[float], xe: List[float], centered: List[bool],
             fixed: bool, epsilon: float, gamma: int, fcycle: bool, skip_pre: bool, nu1: int, nu2: int,
             max_iters_outer: int, stop: str, rtol: float, precision: str, inner_cycles: int,
             outer: str) -> Tuple[torch.Tensor, torch.Tensor]:
    opts = (fixed, epsilon, gamma, fcycle, skip_pre, nu1, nu2, max_iters_outer, stop, rtol, precision, inner_cycles,
            outer)
    return _run(_grids(m, xb, xe, centered), phi0, rhs, lam, (D_xx, D_yy), D_xy, opts)


@solve_2d.register_fake
def _solve_2d_fake(phi0, rhs, lam, D_xx, D_yy, D_xy, m, xb, xe, centered, *opts):
    return torch.empty_like(phi0), phi0.new_empty((), dtype=torch.int64)


@torch.library.custom_op("jmg::solve_3d", mutates_args=())
def solve_3d(phi0: torch.Tensor, rhs: torch.Tensor, lam: torch.Tensor, D_xx: torch.Tensor, D_yy: torch.Tensor,
             D_zz: torch.Tensor, m: List[int], xb: List[float], xe: List[float], centered: List[bool],
             fixed: bool, epsilon: float, gamma: int, fcycle: bool, skip_pre: bool, nu1: int, nu2: int,
             max_iters_outer: int, stop: str, rtol: float, precision: str, inner_cycles: int,
             outer: str) -> Tuple[torch.Tensor, torch.Tensor]:
    opts = (fixed, epsilon, gamma, fcycle, skip_pre, nu1, nu2, max_iters_outer, stop, rtol, precision, inner_cycles,
            outer)
    return _run(_grids(m, xb, xe, centered), phi0, rhs, lam, (D_xx, D_yy, D_zz), None, opts)


@solve_3d.register_fake
def _solve_3d_fake(phi0, rhs, lam, D_xx, D_yy, D_zz, m, xb, xe, centered, *opts):
    return torch.empty_like(phi0), phi0.new_empty((), dtype=torch.int64)


def grid_args(*grids):
    """Per-axis (m, xb, xe, centered) lists of grid_1D objects, x first."""
    return ([int(g.mx) for g in grids], [float(g.xb) for g in grids], [float(g.xe) for g in grids],
            [bool(g.centered) for g in grids])
