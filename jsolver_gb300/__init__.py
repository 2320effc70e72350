"""jsolver_gb300 — GB300-native (sm_103a) geometric multigrid, drop-in for davef96/jsolver.

Solves div(D grad phi) - lam phi = rhs on jsolver's padded Cartesian grids with the
reference's red-black Gauss-Seidel multigrid (V/W/F cycles, fixed and dynamic modes).
Modules mirror the reference package: ``grid_1d``, ``solver_2d``, ``solver_3d``,
``boundary_handler_2d``, ``boundary_handler_3d``. The compute runs in ``libjmg.so``
(CUDA, C ABI in include/jmg.h).
"""
from .grid_1d import grid_1D  # noqa: F401

__all__ = ["grid_1D"]
