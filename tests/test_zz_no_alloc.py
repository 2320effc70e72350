"""jmg_rel_residual_noalloc: the residual measure for callers that cannot allocate.

Some callers cannot allocate device memory: a server that has reserved the whole device
heap for its own pool, a plugin host that passes only inputs and outputs, a loop that
cannot afford the synchronisation an allocation may cause. For them the library offers
jmg_rel_residual_noalloc, whose scratch is a fixed array of the library's own device
memory instead of a caller workspace. This test calls it through the C ABI and checks it
against jmg_rel_residual (which uses a caller workspace) on consecutive calls with
different grids and coefficient forms (arrays and scalars, a phi with a nonzero frame, a
3D grid large enough for the wide reduction), so a call that read stale scratch from the
previous one would fail.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from jsolver_gb300 import _engine, _lib  # noqa: E402
from jsolver_gb300 import workloads as W  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402

DEV = torch.device("cuda", 0)
TOL = 1e-12  # relative, the tolerance of the operator-level parity tests
vp = ctypes.c_void_p


def _dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


def _problem(dim, m, seed, cycles):
    """A partially converged iterate (a few fixed cycles), so the residual is not trivial."""
    from jsolver_gb300.solver_2d import solve_2d
    from jsolver_gb300.solver_3d import solve_3d
    if dim == 2:
        p = W.random_2d(m, seed=seed)
        g = grid_1D(m)
        phi, _ = solve_2d(g, g, p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], fixed=True,
                          max_iters_outer=cycles)
        return (g, g), phi, p["rhs"], p["lam"], (p["D_xx"], p["D_yy"])
    p = W.random_3d(m, seed=seed)
    g = grid_1D(m)
    phi, _ = solve_3d(g, g, g, p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"], fixed=True,
                      max_iters_outer=cycles)
    return (g, g, g), phi, p["rhs"], p["lam"], (p["D_xx"], p["D_yy"], p["D_zz"])


def _coeffs(lam, D):
    """JmgCoeffs over device copies; a Python float selects the scalar form."""
    keep = []
    co = _lib.JmgCoeffs()
    if np.ndim(lam) == 0:
        co.lam, co.lam_scalar = None, float(lam)
    else:
        keep.append(_dev(lam))
        co.lam = keep[-1].data_ptr()
    for k, d in enumerate(D):
        if np.ndim(d) == 0:
            co.D[k], co.D_scalar[k] = None, float(d)
        else:
            keep.append(_dev(d))
            co.D[k] = keep[-1].data_ptr()
    return co, keep


def _random_case(ms, seed, scalar_D=False, scalar_lam=False, frame=False):
    """Random phi and rhs (a nontrivial residual) on grids of resolutions ms = (mx, my[, mz]);
    with frame=True, the frames of phi and rhs hold random values too (both entry points
    read phi's frame as 0 and rhs at interior points only)."""
    rng = np.random.default_rng(seed)
    shape = tuple(m + 3 for m in reversed(ms))
    phi = rng.standard_normal(shape)
    rhs = rng.standard_normal(shape)
    if not frame:
        phi, rhs = W._zero_frame(phi), W._zero_frame(rhs)
    D = tuple(1.0 + 0.5 * k for k in range(len(ms))) if scalar_D else \
        tuple(np.exp(rng.standard_normal(shape)) for _ in ms)
    lam = 0.75 if scalar_lam else rng.uniform(0.0, 5.0, shape)
    return tuple(grid_1D(m) for m in ms), phi, rhs, lam, D


def _with_workspace(grids, phi, rhs, co):
    lib = _lib.load()
    plan = _lib.Plan(_engine.make_grid(grids), _engine.make_config())
    ws = torch.empty(plan.workspace_bytes, dtype=torch.uint8, device=DEV)
    plan_co = _lib.JmgCoeffs.from_buffer_copy(co)
    _lib.check(lib.jmg_build_hierarchy(plan.handle, ctypes.byref(plan_co), vp(ws.data_ptr()),
                                       ctypes.c_size_t(ws.numel()), vp(torch.cuda.current_stream().cuda_stream)))
    out = torch.empty((), dtype=torch.float64, device=DEV)
    _lib.check(lib.jmg_rel_residual(plan.handle, vp(phi.data_ptr()), vp(rhs.data_ptr()), vp(out.data_ptr()),
                                    vp(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                    vp(torch.cuda.current_stream().cuda_stream)))
    return float(out.item())


def _no_alloc(grids, phi, rhs, co):
    lib = _lib.load()
    grid = _engine.make_grid(grids)
    out = torch.full((), float("nan"), dtype=torch.float64, device=DEV)
    rc = lib.jmg_rel_residual_noalloc(ctypes.byref(grid), vp(phi.data_ptr()), vp(rhs.data_ptr()), ctypes.byref(co),
                                      vp(out.data_ptr()), vp(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc)
    return float(out.item())


def test_no_alloc_matches_workspace_version_on_consecutive_calls():
    """Consecutive calls on different grids and coefficient forms share the one scratch
    array; each must match jmg_rel_residual, and repeating the first call must give the
    same bits after the others have overwritten the scratch."""
    cases = [
        lambda: _problem(2, 256, 1, 3),                                   # array lam and D
        lambda: _problem(3, 32, 2, 2),
        lambda: _random_case((64, 64), 3, scalar_D=True),                # scalar D, array lam
        lambda: _random_case((128, 64), 4, scalar_lam=True),             # array D, scalar lam
        lambda: _random_case((16, 32, 16), 5, scalar_D=True, scalar_lam=True),
        lambda: _random_case((32, 32, 32), 6, scalar_D=True),
        lambda: _random_case((256, 256), 7, frame=True),                 # phi's frame is not zero
        lambda: _random_case((16, 16, 32), 8, frame=True, scalar_lam=True),
        lambda: _random_case((32, 128, 64), 9),  # 127 x 63 = 8001 interior rows: 1216 partial sums
        lambda: _problem(2, 256, 1, 3),
    ]
    results = []
    for make in cases:
        grids, phi, rhs, lam, D = make()
        co, keep = _coeffs(lam, D)
        phi_d, rhs_d = _dev(phi), _dev(rhs)
        want = _with_workspace(grids, phi_d, rhs_d, co)
        got = _no_alloc(grids, phi_d, rhs_d, co)
        assert np.isfinite(got) and want > 0
        assert abs(got - want) <= TOL * want, ([g.mx for g in grids], got, want)
        results.append(got)
    # the repeated first case gives the same value after other grids used the scratch
    assert results[0] == results[-1]


def test_no_alloc_rejects_d_xy_in_3d():
    lib = _lib.load()
    g = grid_1D(8)
    grid = _engine.make_grid((g, g, g))
    x = torch.zeros((11, 11, 11), dtype=torch.float64, device=DEV)
    co = _lib.JmgCoeffs()
    for k in range(3):
        co.D[k] = x.data_ptr()
    co.lam = x.data_ptr()
    co.D_xy = x.data_ptr()
    out = torch.zeros((), dtype=torch.float64, device=DEV)
    rc = lib.jmg_rel_residual_noalloc(ctypes.byref(grid), vp(x.data_ptr()), vp(x.data_ptr()), ctypes.byref(co),
                                      vp(out.data_ptr()), vp(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.JMG_ERR_VALUE
    assert b"D_xy is a 2D argument" in lib.jmg_last_error()


def test_no_alloc_rejects_grids_beyond_its_scratch():
    lib = _lib.load()
    g = grid_1D(1024)
    grid = _engine.make_grid((g, g))
    co = _lib.JmgCoeffs()
    co.lam_scalar = 0.0
    co.D_scalar[0] = co.D_scalar[1] = 1.0
    x = torch.zeros((1027, 1027), dtype=torch.float64, device=DEV)
    out = torch.zeros((), dtype=torch.float64, device=DEV)
    rc = lib.jmg_rel_residual_noalloc(ctypes.byref(grid), vp(x.data_ptr()), vp(x.data_ptr()), ctypes.byref(co),
                                      vp(out.data_ptr()), vp(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.JMG_ERR_VALUE
    assert b"limit" in lib.jmg_last_error()
