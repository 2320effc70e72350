"""Host-side behaviour of the public API: the reference's errors, wrappers, defaults.

Everything here runs without a GPU: grid validation happens when the plan is created
(libjmg, host code) and dtype/shape validation in Python, both before any device work
(the reference's order: Solver_2D.__init__ checks, then solve's checks,
solver_2d.py:276-277, 449-453)."""
import inspect

import numpy as np
import pytest
import torch

from jsolver_gb300 import solver_2d as s2
from jsolver_gb300 import solver_3d as s3
from jsolver_gb300.grid_1d import grid_1D

Z = np.zeros(131)


@pytest.mark.parametrize("gx,gy,msg", [
    (128, 100, "Resolution of y-grid is not a power of 2. Value: 100"),
    (100, 128, "Resolution of x-grid is not a power of 2. Value: 100"),
    (128, 4, "Resolution of x-grid not efficient for multigrid configuration. Resolution of coarsest level: 32"),
    (4, 128, "Resolution of y-grid not efficient for multigrid configuration. Resolution of coarsest level: 32"),
])
def test_2d_grid_errors(gx, gy, msg):
    with pytest.raises(ValueError) as e:
        s2.solve_2d_simple(grid_x=grid_1D(mx=gx), grid_y=grid_1D(mx=gy), phi=Z, rhs=Z, lam=Z, D_xx=1.0, D_yy=1.0)
    assert str(e.value) == msg


def test_2d_linear_grid_error():
    for gx, gy in ((grid_1D(128), grid_1D(128, grid_type=1)), (grid_1D(128, grid_type=1), grid_1D(128))):
        with pytest.raises(ValueError, match="Only linear grids are supported!"):
            s2.solve_2d_simple(grid_x=gx, grid_y=gy, phi=Z, rhs=Z, lam=Z, D_xx=1.0, D_yy=1.0)


@pytest.mark.parametrize("m,axis,kind", [
    ((100, 128, 128), "x", "is not a power of 2"), ((128, 100, 32), "y", "is not a power of 2"),
    ((128, 32, 55), "z", "is not a power of 2"),
    ((32, 4, 4), "x", "not efficient for multigrid configuration"),
    ((4, 32, 4), "y", "not efficient for multigrid configuration"),
    ((4, 4, 32), "z", "not efficient for multigrid configuration")])
def test_3d_grid_errors(m, axis, kind):
    """tests/test_solver_3d.py:85-118 check these substrings."""
    with pytest.raises(ValueError) as e:
        s3.solve_3d_simple(grid_x=grid_1D(m[0]), grid_y=grid_1D(m[1]), grid_z=grid_1D(m[2]), phi=Z, rhs=Z, lam=Z,
                           D_xx=1.0, D_yy=1.0, D_zz=1.0)
    assert f"Resolution of {axis}-grid {kind}" in str(e.value)


@pytest.mark.parametrize("which", [0, 1, 2])
def test_3d_linear_error(which):
    gs = [grid_1D(32), grid_1D(32), grid_1D(32)]
    gs[which] = grid_1D(32, grid_type=1)
    with pytest.raises(ValueError, match="Only linear grids are supported"):
        s3.solve_3d_simple(*gs, phi=Z, rhs=Z, lam=Z, D_xx=1.0, D_yy=1.0, D_zz=1.0)


def test_dtype_error():
    g = grid_1D(16)
    a = np.zeros((19, 19))
    with pytest.raises(ValueError, match="dtype must be 'jnp.float64'"):
        s2.solve_2d_simple(g, g, a.astype(np.float32), a, 0.0, 1.0, 1.0)
    with pytest.raises(ValueError, match="dtype must be 'jnp.float64'"):
        s2.solve_2d_simple(g, g, a, a, 0, 1.0, 1.0)  # Python int lam traces as int64
    with pytest.raises(ValueError, match="dtype must be 'jnp.float64'"):
        s2.solve_2d_simple(g, g, a, a, 0.0, 1.0, 1.0, D_xy=np.zeros((19, 19), np.float32))


def test_shape_errors():
    g = grid_1D(16)
    a = np.zeros((19, 19))
    with pytest.raises(ValueError, match=r"Shape mismatch: phi=\(19, 19\), rhs=\(19, 18\)"):
        s2.solve_2d_simple(g, g, a, np.zeros((19, 18)), 0.0, 1.0, 1.0)
    with pytest.raises(ValueError, match="Shape mismatch"):
        s2.solve_2d_simple(g, g, a, a, 0.0, a, 1.0)  # D components mixed scalar/array
    with pytest.raises(ValueError, match="Shape mismatch"):
        s2.solve_2d_simple(g, g, a, a, np.zeros((3, 3)), 1.0, 1.0)
    with pytest.raises(ValueError, match="Shape mismatch"):
        s2.solve_2d_simple(g, g, np.zeros((35, 35)), np.zeros((35, 35)), 0.0, 1.0, 1.0)  # not the grid's shape
    g3 = grid_1D(8)
    b = np.zeros((11, 11, 11))
    with pytest.raises(ValueError, match="Shape mismatch.*D_zz="):
        s3.solve_3d_simple(g3, g3, g3, b, b, 0.0, b, b, 1.0)


def test_batched_shape_errors_and_no_gpu(monkeypatch):
    """Batched solves: (B, *spatial) phi/rhs, coefficients shared or (B, *spatial); the
    per-problem rules are the single solve's; without a device the call raises."""
    g = grid_1D(16)
    a = np.zeros((3, 19, 19))
    with pytest.raises(ValueError, match=r"batched phi and rhs must both have shape \(B, 19, 19\)"):
        s2.solve_2d_batched(g, g, a[0], a[0], 0.0, 1.0, 1.0)
    with pytest.raises(ValueError, match="batched phi and rhs"):
        s2.solve_2d_batched(g, g, a, a[:2], 0.0, 1.0, 1.0)
    with pytest.raises(ValueError, match="batch of 3"):
        s2.solve_2d_batched(g, g, a, a, np.zeros((2, 19, 19)), 1.0, 1.0)
    with pytest.raises(ValueError, match="Shape mismatch"):
        s2.solve_2d_batched(g, g, a, a, 0.0, a[0], 1.0)  # D components mixed scalar/array
    with pytest.raises(ValueError, match="dtype must be 'jnp.float64'"):
        s2.solve_2d_batched(g, g, a.astype(np.float32), a, 0.0, 1.0, 1.0)
    g3 = grid_1D(8)
    b = np.zeros((2, 11, 11, 11))
    with pytest.raises(ValueError, match="Shape mismatch.*D_zz="):
        s3.solve_3d_batched(g3, g3, g3, b, b, 0.0, b, b, 1.0)
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(RuntimeError, match="CUDA"):
        s2.solve_2d_batched(g, g, a, a, 0.0, 1.0, 1.0)


def test_no_gpu_fails_loudly(monkeypatch):
    """With valid arguments and no CUDA device the call raises; it never computes on the CPU."""
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    g = grid_1D(16)
    a = np.zeros((19, 19))
    with pytest.raises(RuntimeError, match="CUDA"):
        s2.solve_2d_simple(g, g, a, a, 0.0, 1.0, 1.0)


def test_wrappers_complete_and_positional():
    # the reference's 18 wrappers per dimension; solve_*d_batched is this package's extension
    names2 = sorted(n for n in dir(s2) if n.startswith("solve_2d_") and n != "solve_2d_batched")
    names3 = sorted(n for n in dir(s3) if n.startswith("solve_3d_") and n != "solve_3d_batched")
    assert len(names2) == len(names3) == 18
    for suffix in ("", "_skip_pre", "_fcycle", "_fcycle_skip_pre", "_wcycle", "_wcycle_skip_pre"):
        assert list(inspect.signature(getattr(s2, f"solve_2d{suffix}_simple")).parameters)[:8] == \
            ["grid_x", "grid_y", "phi", "rhs", "lam", "D_xx", "D_yy", "D_xy"]
        assert list(inspect.signature(getattr(s2, f"solve_2d_fixed{suffix}_simple")).parameters)[:3] == \
            ["grid_x", "grid_y", "iters"]
        assert list(inspect.signature(getattr(s2, f"solve_2d_fixed{suffix}")).parameters)[:4] == \
            ["grid_x", "grid_y", "iters_outer", "iters_inner"]
        assert list(inspect.signature(getattr(s3, f"solve_3d{suffix}_simple")).parameters)[:9] == \
            ["grid_x", "grid_y", "grid_z", "phi", "rhs", "lam", "D_xx", "D_yy", "D_zz"]


def test_solve_signature_defaults():
    sig = inspect.signature(s2.solve_2d)
    d = {k: v.default for k, v in sig.parameters.items() if v.default is not inspect.Parameter.empty}
    assert d["fixed"] is False and d["epsilon"] == 1e-12 and d["gamma"] == 1 and d["fcycle"] is False
    assert d["skip_pre"] is False and d["nu1"] == 1 and d["nu2"] == 1
    assert d["max_iters_outer"] == d["max_iters_inner"] == 2 ** 31 - 1
    assert d["D_xy"] is None


def test_solver_class_shapes():
    s = s2.Solver_2D(grid_1D(64), grid_1D(128))
    assert s.levels == 7 and s.arr_shape[0] == (131, 67) and s.arr_shape[-1] == (5, 4)
    t = s3.Solver_3D(grid_1D(32), grid_1D(64), grid_1D(32))
    assert t.levels == 6 and t.arr_shape[0] == (35, 67, 35)
