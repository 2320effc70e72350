"""jmg_rel_residual_noalloc: the residual measure for callers that cannot allocate.

Some callers cannot allocate device memory: a server that has reserved the whole device
heap for its own pool, a plugin host that passes only inputs and outputs, a loop that
cannot afford the synchronisation an allocation may cause. For them the library offers
jmg_rel_residual_noalloc, whose scratch is a fixed array of the library's own device
memory instead of a caller workspace. This test calls it through the C ABI and checks it
against jmg_rel_residual (which uses a caller workspace) on consecutive calls with
different grids, so a call that read stale scratch from the previous one would fail.
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
    keep = [_dev(lam)] + [_dev(d) for d in D]
    co = _lib.JmgCoeffs()
    co.lam = keep[0].data_ptr()
    for k, t in enumerate(keep[1:]):
        co.D[k] = t.data_ptr()
    return co, keep


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
    cases = [(2, 256, 1, 3), (3, 32, 2, 2), (2, 64, 3, 1), (2, 256, 1, 3)]
    results = []
    for dim, m, seed, cycles in cases:
        grids, phi, rhs, lam, D = _problem(dim, m, seed, cycles)
        co, keep = _coeffs(lam, D)
        phi_d, rhs_d = _dev(phi), _dev(rhs)
        want = _with_workspace(grids, phi_d, rhs_d, co)
        got = _no_alloc(grids, phi_d, rhs_d, co)
        assert np.isfinite(got) and want > 0
        assert abs(got - want) <= TOL * want, (dim, m, got, want)
        results.append(got)
    # the repeated first case gives the same value after other grids used the scratch
    assert results[0] == results[3]


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
