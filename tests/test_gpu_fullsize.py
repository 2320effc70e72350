"""GPU parity at the benchmark sizes: 2D 1024^2 and 3D 256^3 random-coefficient problems.

No tuning variable is set, so the paths the solver picks by itself at these sizes run:
  * 2D 1024^2: 11 levels, grid-wide kernels down to 64^2 and the single-block coarse
    kernel from 32^2 (the 2048-point threshold);
  * 3D 256^3: the one-pass FP32 sweep on the level-0 FP32 arrays of mixed solves (levels
    that fill half a wave), the tiled restriction and cell prolongation, 1216-block
    residual reductions (more than 4096 interior rows) and 608-block FCG kernels.

Fixed-count solves are compared with the C oracle (the reference's fixed loop,
solver_2d.py:461-463 / solver_3d.py:468-470) at 1e-12 relative L2, the bar of every
full-solve parity test. The one-pass sweep must give the same bits as the colour passes
(JMG_FUSED=0) in a whole mixed solve. The headline forms must meet the relative residual
1e-10 measured by the NumPy oracle in FP64 (up to the FCG recurrence's drift, 2e-10).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from jsolver_gb300 import _engine  # noqa: E402
from jsolver_gb300 import workloads as W  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d  # noqa: E402
from jsolver_gb300.solver_3d import solve_3d  # noqa: E402
from oracle import c_oracle, mg2d, mg3d  # noqa: E402

TUNING = ("JMG_HOST_LOOP", "JMG_PDL", "JMG_COARSE_POINTS", "JMG_COARSE", "JMG_COARSE32", "JMG_FUSED", "JMG_FUSED2D",
          "JMG_FUSED64", "JMG_FUSED_POINTS", "JMG_RESTRICT3D", "JMG_PROLONG3D", "JMG_PROLONG2D", "JMG_FCG_BLOCKS",
          "JMG_ADJ_BLOCK_POINTS", "JMG_COARSE_OPS", "JMG_FUSEDOPS", "JMG_FUSEDOPS_MAX", "JMG_COARSE_THREADS",
          "JMG_COARSE_WARP", "JMG_MID", "JMG_MID_POINTS", "JMG_MID_STALL", "JMG_SWEEP3D")


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(autouse=True)
def _defaults(monkeypatch):
    """Every case runs with the solver's own choices (no tuning variable, fresh plans)."""
    for k in TUNING:
        monkeypatch.delenv(k, raising=False)
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())


@pytest.fixture(scope="module")
def p2d():
    p = W.random_2d(1024, seed=0)
    return (grid_1D(1024),) * 2, (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"]), p


@pytest.fixture(scope="module")
def p3d():
    p = W.random_3d(256, seed=0)
    return (grid_1D(256),) * 3, (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"]), p


@pytest.mark.parametrize("cycles,form", [(4, {}), (2, {"gamma": 2})], ids=["V4", "W2"])
def test_2d_1024_fixed_cycles_match_oracle(p2d, cycles, form):
    grids, args, _ = p2d
    phi, c = solve_2d(*grids, *args, fixed=True, max_iters_outer=cycles, **form)
    ref, _, _ = c_oracle.solve(grids, args[0], args[1], args[2], args[3:], fixed=True, max_iters_outer=cycles, **form)
    assert c == cycles
    assert rel_l2(phi, ref) < 1e-12, rel_l2(phi, ref)


def test_2d_1024_residual_stop_count_matches_oracle(p2d):
    """The reference's stationary FP64 iteration to rel. residual 1e-10: same cycle count
    as the oracle (271 on this problem) and the same phi."""
    grids, args, _ = p2d
    phi, c = solve_2d(*grids, *args, stop="residual", rtol=1e-10)
    ref, rc, rr = c_oracle.solve(grids, args[0], args[1], args[2], args[3:], stop="residual", rtol=1e-10)
    assert c == rc and rr <= 1e-10
    assert rel_l2(phi, ref) < 1e-12, rel_l2(phi, ref)


def test_3d_256_fixed_f_cycles_match_oracle(p3d):
    grids, args, _ = p3d
    phi, c = solve_3d(*grids, *args, fixed=True, max_iters_outer=2, fcycle=True)
    ref, _, _ = c_oracle.solve(grids, args[0], args[1], args[2], args[3:], fixed=True, max_iters_outer=2, fcycle=True)
    assert rel_l2(phi, ref) < 1e-12, rel_l2(phi, ref)


def test_3d_256_onepass_fp32_sweep_bit_identical(p3d, monkeypatch):
    """Mixed solve (FP32 cycles whose level-0 sweeps run in one pass at this size) against
    the same solve with colour passes only: the same bits."""
    grids, args, _ = p3d
    kw = dict(precision="mixed", fixed=True, max_iters_outer=3, fcycle=True)
    phi_a, _ = solve_3d(*grids, *args, **kw)
    monkeypatch.setenv("JMG_FUSED", "0")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_b, _ = solve_3d(*grids, *args, **kw)
    np.testing.assert_array_equal(phi_a, phi_b)


def test_3d_256_tma_sweep_equals_register_sweep(p3d, monkeypatch):
    """The same mixed solve with the level-0 one-pass sweep fed by TMA copies (the default)
    and by register loads (JMG_SWEEP3D=regs): the same bits."""
    grids, args, _ = p3d
    kw = dict(precision="mixed", fixed=True, max_iters_outer=3, fcycle=True)
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_a, _ = solve_3d(*grids, *args, **kw)
    monkeypatch.setenv("JMG_SWEEP3D", "regs")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_b, _ = solve_3d(*grids, *args, **kw)
    np.testing.assert_array_equal(phi_a, phi_b)


@pytest.mark.parametrize("form", [dict(inner_cycles=2), dict(nu2=5, inner_cycles=1)], ids=["V11x2", "V15x1"])
def test_2d_1024_headline_form_reaches_rtol(p2d, form):
    """The mixed + FCG form with two V(1,1) cycles per step and with one V(1,5) cycle per
    step (bench.py's fast form; its extra post-sweeps run as one-pass launches): the
    oracle's FP64 residual meets the tolerance."""
    grids, args, p = p2d
    phi, c = solve_2d(*grids, *args, stop="residual", rtol=1e-10, precision="mixed", outer="fcg", **form)
    o = mg2d.Oracle2D(*grids)
    o.setup(*args)
    assert o.rel_residual(phi, p["rhs"]) <= 2e-10
    assert rel_l2(phi, p["phi_exact"]) < 1e-6
    assert int(c) < 60


@pytest.mark.parametrize("form", [dict(inner_cycles=2), dict(nu2=3, inner_cycles=1)], ids=["F11x2", "F13x1"])
def test_3d_256_headline_form_reaches_rtol(p3d, form):
    """The same for 3D F-cycles: two F(1,1) or one F(1,3) cycle per FCG step."""
    grids, args, p = p3d
    phi, c = solve_3d(*grids, *args, stop="residual", rtol=1e-10, precision="mixed", outer="fcg", fcycle=True,
                      **form)
    o = mg3d.Oracle3D(*grids)
    o.setup(*args)
    assert o.rel_residual(phi, p["rhs"]) <= 2e-10
    assert int(c) < 100
