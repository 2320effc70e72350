"""The persistent middle-level kernel (mg_mid2d.cu) against the separate launches.

With JMG_MID=1 a 2D plan runs its levels of at most 2^19 padded points, together with
the coarse sub-cycle, in one cooperative launch: the fused operator pairs spread over one
block per SM with grid barriers between them, the coarse levels on block 0 in shared
memory. Every value comes from the same per-point functions in the same order, so whole
solves must match the separate launches (the default) bit for bit, in every cycle shape
(V, W, F, F with gamma 2), sweep count, precision and outer iteration. The colour-pass
solves are checked against the oracle in test_gpu_parity.py and test_gpu_fullsize.py.

The barrier waits are bounded. JMG_MID_STALL=1 (with JMG_MID=1) makes the first barrier
of each launch expect one block more than there are, so its wait always runs out: the
solve must end early with JMG_ERR_TIMEOUT from jmg_solve_check (the host-input API
raises), and the next solve on a fresh plan must give the right answer, i.e. the context
stays usable.
"""
import ctypes
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from jsolver_gb300 import _engine, _lib  # noqa: E402
from jsolver_gb300 import workloads as W  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d  # noqa: E402

DEV = torch.device("cuda", 0)
ENV = ("JMG_MID", "JMG_MID_POINTS", "JMG_MID_STALL", "JMG_FUSEDOPS")


def _args(mx, my, seed):
    p = W.random_2d(max(mx, my), seed=seed)
    sl = (slice(0, my + 3), slice(0, mx + 3))
    args = [torch.from_numpy(np.ascontiguousarray(p[k][sl])).to(DEV) for k in ("phi0", "rhs", "lam", "D_xx", "D_yy")]
    args[1] = args[1].clone()
    args[1][-2:, :] = 0  # the frame where the slice cut the field
    args[1][:, -2:] = 0
    return args


def _run(monkeypatch, env, grids, args, **opts):
    for k in ENV:
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    _engine.CACHE.plans.clear()
    _engine.CACHE.ws.clear()
    phi, count = solve_2d(*grids, *args, **opts)
    cfg = _engine.make_config(**opts)
    plan = _engine.CACHE.plan(_engine.make_grid(grids), cfg)
    return phi, count, _lib.load().jmg_plan_mid_start(plan.handle)


CASES = [
    ((1024, 1024), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2)),
    ((256, 256), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2)),
    ((512, 512), dict(stop="residual", outer="fcg")),
    ((256, 256), dict(precision="mixed", stop="residual")),
    ((128, 256), dict(precision="mixed", fixed=True, max_iters_outer=6, gamma=2)),
    ((1024, 1024), dict(fixed=True, max_iters_outer=2, gamma=2)),
    ((256, 128), dict(fixed=True, max_iters_outer=5, nu1=2, nu2=1)),
    ((256, 256), dict(fixed=True, max_iters_outer=5, nu1=1, nu2=3)),
    ((256, 256), dict(precision="mixed", fixed=True, max_iters_outer=4, nu1=3, nu2=2)),
    ((256, 256), dict(fixed=True, max_iters_outer=5, skip_pre=True, fcycle=True)),
    ((256, 256), dict(fixed=True, max_iters_outer=4, fcycle=True, gamma=2)),
    ((512, 512), dict(precision="mixed", stop="residual", outer="fcg", fcycle=True)),
    ((64, 256), dict(fixed=True, max_iters_outer=3)),
    ((128, 128), dict()),
]


@pytest.mark.parametrize("shape,opts", CASES, ids=lambda x: str(x))
def test_mid_kernel_equals_separate_launches(monkeypatch, shape, opts):
    mx, my = shape
    grids = (grid_1D(mx), grid_1D(my))
    args = _args(mx, my, seed=3 * mx + my)
    ref, c_ref, m_ref = _run(monkeypatch, {}, grids, args, **opts)
    got, c_got, m_got = _run(monkeypatch, {"JMG_MID": "1"}, grids, args, **opts)
    assert m_ref == -1
    assert m_got >= 1, "the plan did not take the middle-level kernel"
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)


def test_mid_kernel_from_lower_levels(monkeypatch):
    """A smaller JMG_MID_POINTS starts the kernel further down: the same bits."""
    grids = (grid_1D(512), grid_1D(512))
    args = _args(512, 512, seed=11)
    opts = dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2)
    ref, c_ref, _ = _run(monkeypatch, {}, grids, args, **opts)
    # padded points per level: 515^2, 259^2, 131^2 = 17161, 67^2 = 4489; coarse block from 35^2
    for pts, lev in (("20000", 2), ("5000", 3)):
        got, c_got, m = _run(monkeypatch, {"JMG_MID": "1", "JMG_MID_POINTS": pts}, grids, args, **opts)
        assert m == lev
        assert int(c_got) == int(c_ref)
        assert torch.equal(got, ref)


def test_mid_kernel_host_loop(monkeypatch):
    """The host-driven loop (profiling mode) launches the same kernel directly."""
    grids = (grid_1D(256), grid_1D(256))
    args = _args(256, 256, seed=5)
    opts = dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2)
    ref, c_ref, _ = _run(monkeypatch, {}, grids, args, **opts)
    monkeypatch.setenv("JMG_HOST_LOOP", "1")
    got, c_got, m = _run(monkeypatch, {"JMG_MID": "1"}, grids, args, **opts)
    assert m >= 1
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("opts", [dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2),
                                  dict(stop="residual"), dict(fixed=True, max_iters_outer=50, gamma=2)],
                         ids=["mixed-fcg", "fp64-dynamic", "fp64-fixed-W"])
def test_barrier_timeout_is_reported_and_context_survives(monkeypatch, opts):
    grids = (grid_1D(256), grid_1D(256))
    args = _args(256, 256, seed=9)
    ref, c_ref, _ = _run(monkeypatch, {}, grids, args, **opts)
    # host inputs: the API checks the workspace's fault flag and raises
    host = [a.cpu().numpy() for a in args]
    t0 = time.time()
    with pytest.raises(RuntimeError, match="jmg error 4"):
        _run(monkeypatch, {"JMG_MID": "1", "JMG_MID_STALL": "1"}, grids, host, **opts)
    assert time.time() - t0 < 60  # the loop ends at the first run-out wait, not at its cycle limit
    # device inputs: the result is void (NaN) and jmg_solve_check says why
    got, _, m = _run(monkeypatch, {"JMG_MID": "1", "JMG_MID_STALL": "1"}, grids, args, **opts)
    assert m >= 1
    cfg = _engine.make_config(**opts)
    plan = _engine.CACHE.plan(_engine.make_grid(grids), cfg)
    ws = _engine.CACHE.workspace(plan, DEV)
    rc = _lib.load().jmg_solve_check(plan.handle, ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                     ctypes.c_void_p(torch.cuda.current_stream(DEV).cuda_stream))
    assert rc == _lib.JMG_ERR_TIMEOUT
    assert "ran out" in _lib.load().jmg_last_error().decode()
    assert torch.isnan(got).any()
    # the next solve on a fresh plan, same context: the right answer, and the check passes
    again, c_again, _ = _run(monkeypatch, {"JMG_MID": "1"}, grids, args, **opts)
    assert int(c_again) == int(c_ref)
    assert torch.equal(again, ref)
    plan = _engine.CACHE.plan(_engine.make_grid(grids), cfg)
    ws = _engine.CACHE.workspace(plan, DEV)
    assert _lib.load().jmg_solve_check(plan.handle, ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                       ctypes.c_void_p(torch.cuda.current_stream(DEV).cuda_stream)) == 0
