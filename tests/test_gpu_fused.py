"""One-pass sweeps (mg_fused.cu, 3D and 2D) and the tiled 3D restriction (mg_tile3d.cu)
against the two colour passes and the one-thread-per-coarse-point restriction.

The one-pass sweep computes every value with the colour passes' arithmetic in the same
order, so whole solves must agree bit for bit with the one-pass sweep switched off
(JMG_FUSED=0), for every cycle shape, sweep count and grid shape, in FP32 cycles and
in FP64; the colour-pass solves are checked against the oracle in test_gpu_parity.py.
The environment switches are read when a plan is created, so every case builds new plans.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from jsolver_gb300 import _engine  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_3d import solve_3d  # noqa: E402

DEV = torch.device("cuda", 0)


def _problem(mx, my, mz, seed):
    rng = np.random.default_rng(seed)
    shp = (mz + 3, my + 3, mx + 3)

    def field(scale):
        a = rng.standard_normal(shp) * scale
        a[:2], a[-1:], a[:, :2], a[:, -1:], a[:, :, :2], a[:, :, -1:] = 0, 0, 0, 0, 0, 0
        return a

    D = [np.exp(field(0.7)) for _ in range(3)]
    lam = np.abs(field(3.0))
    rhs = field(1.0)
    return [torch.from_numpy(x).to(DEV) for x in [np.zeros(shp), rhs, lam] + D]


def _solve(monkeypatch, env, grids, args, **opts):
    for k in ("JMG_FUSED", "JMG_FUSED64", "JMG_FUSED_POINTS", "JMG_RESTRICT3D", "JMG_FUSED2D", "JMG_PROLONG3D",
                  "JMG_PROLONG2D", "JMG_SWEEP3D"):
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    _engine.CACHE.plans.clear()
    _engine.CACHE.ws.clear()
    return solve_3d(*grids, *args, **opts)


CASES = [
    ((64, 64, 64), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2, fcycle=True)),
    ((64, 64, 64), dict(precision="mixed", stop="residual")),
    ((64, 32, 128), dict(precision="mixed", stop="residual", outer="fcg")),
    ((128, 64, 32), dict(precision="mixed", fixed=True, max_iters_outer=6, gamma=2)),
    ((64, 64, 64), dict(precision="mixed", fixed=True, max_iters_outer=5, nu1=2, nu2=1)),
    ((64, 64, 64), dict(precision="mixed", fixed=True, max_iters_outer=5, skip_pre=True)),
    ((32, 64, 64), dict(fixed=True, max_iters_outer=4, fcycle=True)),
    ((64, 64, 64), dict()),
]


@pytest.mark.parametrize("shape,opts", CASES)
def test_one_pass_equals_colour_passes(monkeypatch, shape, opts):
    grids = tuple(grid_1D(m) for m in shape)
    args = _problem(*shape, seed=sum(shape))
    ref, c_ref = _solve(monkeypatch, {"JMG_FUSED": "0"}, grids, args, **opts)
    # every level of at least 4096 points sweeps in one pass, FP32 and FP64
    got, c_got = _solve(monkeypatch, {"JMG_FUSED_POINTS": "4096", "JMG_FUSED64": "1"}, grids, args, **opts)
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("shape,opts", CASES[:6] + [
    ((32, 64, 128), dict(precision="mixed", fixed=True, max_iters_outer=4)),
    ((128, 128, 64), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2, fcycle=True))])
def test_tma_sweep_equals_register_sweep(monkeypatch, shape, opts):
    """FP32 one-pass sweeps with their plane tiles fed by TMA copies (mg_sweep_tma3d.cu,
    the default) and by register loads (k_sweep_fused3d, JMG_SWEEP3D=regs), on every level
    of at least 4096 points: the same bits. On these small levels the blocks' work ranges
    cut the tiles' plane columns at arbitrary planes, so the march's restart at a tile
    boundary is covered too."""
    grids = tuple(grid_1D(m) for m in shape)
    args = _problem(*shape, seed=3 + sum(shape))
    ref, c_ref = _solve(monkeypatch, {"JMG_FUSED_POINTS": "4096", "JMG_SWEEP3D": "regs"}, grids, args, **opts)
    got, c_got = _solve(monkeypatch, {"JMG_FUSED_POINTS": "4096"}, grids, args, **opts)
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("shape,opts", [CASES[0], CASES[2], CASES[6], CASES[7],
                                        ((64, 64, 32), dict(fixed=True, max_iters_outer=3, nu1=1, nu2=0))])
def test_tiled_restriction_equals_grid_restriction(monkeypatch, shape, opts):
    """The same solves with the tiled 3D restriction and the cell prolongation (defaults)
    and with the grid-wide ones (nu2 = 0 makes the prolongation bilinear)."""
    grids = tuple(grid_1D(m) for m in shape)
    args = _problem(*shape, seed=7 + sum(shape))
    ref, c_ref = _solve(monkeypatch, {"JMG_RESTRICT3D": "grid", "JMG_PROLONG3D": "grid"}, grids, args, **opts)
    got, c_got = _solve(monkeypatch, {}, grids, args, **opts)
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)


CASES_2D = [
    ((256, 256), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2)),
    ((256, 256), dict(precision="mixed", stop="residual")),
    ((128, 256), dict(precision="mixed", fixed=True, max_iters_outer=6, gamma=2)),
    ((256, 128), dict(fixed=True, max_iters_outer=5, nu1=2, nu2=1)),
    ((256, 256), dict(fixed=True, max_iters_outer=5, skip_pre=True, fcycle=True)),
    ((256, 256), dict()),
]


@pytest.mark.parametrize("shape,opts", CASES_2D)
def test_one_pass_2d_equals_colour_passes(monkeypatch, shape, opts):
    from jsolver_gb300 import workloads as W
    from jsolver_gb300.solver_2d import solve_2d
    mx, my = shape
    p = W.random_2d(max(mx, my), seed=mx + 3 * my)
    sl = (slice(0, my + 3), slice(0, mx + 3))
    args = [torch.from_numpy(np.ascontiguousarray(p[k][sl])).to(DEV) for k in ("phi0", "rhs", "lam", "D_xx", "D_yy")]
    args[1] = args[1].clone()
    args[1][-1:, :] = 0  # a frame of zeros where the slice cut the field
    args[1][:, -1:] = 0
    grids = (grid_1D(mx), grid_1D(my))

    def run(env):
        for k in ("JMG_FUSED", "JMG_FUSED64", "JMG_FUSED_POINTS", "JMG_RESTRICT3D", "JMG_FUSED2D", "JMG_PROLONG3D",
                  "JMG_PROLONG2D"):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        _engine.CACHE.plans.clear()
        _engine.CACHE.ws.clear()
        return solve_2d(*grids, *args, **opts)

    ref, c_ref = run({"JMG_FUSED": "0"})
    # every level of at least 1000 points sweeps in one pass, FP32 and FP64
    got, c_got = run({"JMG_FUSED_POINTS": "1000", "JMG_FUSED64": "1"})
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("shape,opts", [CASES_2D[0], CASES_2D[2], CASES_2D[3],
                                        ((128, 128), dict(fixed=True, max_iters_outer=3, nu1=1, nu2=0))])
def test_cell_prolongation_2d_equals_grid(monkeypatch, shape, opts):
    """2D solves with the cell prolongation (default) and the grid-wide one, bit for bit
    (nu2 = 0 adds the (even, even) points)."""
    from jsolver_gb300 import workloads as W
    from jsolver_gb300.solver_2d import solve_2d
    mx, my = shape
    p = W.random_2d(max(mx, my), seed=2 * mx + my)
    sl = (slice(0, my + 3), slice(0, mx + 3))
    args = [torch.from_numpy(np.ascontiguousarray(p[k][sl])).to(DEV) for k in ("phi0", "rhs", "lam", "D_xx", "D_yy")]
    grids = (grid_1D(mx), grid_1D(my))

    def run(env):
        for k in ("JMG_PROLONG2D",):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        _engine.CACHE.plans.clear()
        _engine.CACHE.ws.clear()
        return solve_2d(*grids, *args, **opts)

    ref, c_ref = run({"JMG_PROLONG2D": "grid"})
    got, c_got = run({})
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)


CASES_OPS = [
    ((256, 256), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2)),
    ((1024, 1024), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2)),
    ((256, 256), dict(precision="mixed", stop="residual")),
    ((512, 512), dict(stop="residual", outer="fcg")),
    ((128, 256), dict(precision="mixed", fixed=True, max_iters_outer=6, gamma=2)),
    ((256, 128), dict(fixed=True, max_iters_outer=5, nu1=2, nu2=1)),
    ((256, 256), dict(fixed=True, max_iters_outer=5, nu1=1, nu2=2)),
    ((256, 256), dict(fixed=True, max_iters_outer=4, nu1=0, nu2=2)),
    ((256, 256), dict(fixed=True, max_iters_outer=4, nu1=2, nu2=0)),
    ((256, 256), dict(fixed=True, max_iters_outer=5, skip_pre=True, fcycle=True)),
    ((256, 256), dict(fixed=True, max_iters_outer=4, fcycle=True, gamma=2)),
    ((64, 256), dict(fixed=True, max_iters_outer=3)),
    ((256, 256), dict()),
]


@pytest.mark.parametrize("shape,opts", CASES_OPS, ids=lambda x: str(x))
def test_fused_operator_pairs_2d_equal_unfused(monkeypatch, shape, opts):
    """2D solves with the fused pairs (smooth + restrict, prolong + smooth over tiles with
    halos; the default on grid-wide 2D levels) and with the separate colour passes,
    tiled restriction and cell prolongation (JMG_FUSEDOPS=0): the same bits and counts,
    in FP64 and FP32 cycles, every cycle shape and sweep count, FCG and Richardson."""
    from jsolver_gb300 import workloads as W
    from jsolver_gb300.solver_2d import solve_2d
    mx, my = shape
    p = W.random_2d(max(mx, my), seed=5 * mx + my)
    sl = (slice(0, my + 3), slice(0, mx + 3))
    args = [torch.from_numpy(np.ascontiguousarray(p[k][sl])).to(DEV) for k in ("phi0", "rhs", "lam", "D_xx", "D_yy")]
    args[1] = args[1].clone()
    args[1][-2:, :] = 0  # the frame where the slice cut the field
    args[1][:, -2:] = 0
    grids = (grid_1D(mx), grid_1D(my))

    def run(env):
        monkeypatch.delenv("JMG_FUSEDOPS", raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        _engine.CACHE.plans.clear()
        _engine.CACHE.ws.clear()
        return solve_2d(*grids, *args, **opts)

    ref, c_ref = run({"JMG_FUSEDOPS": "0"})
    got, c_got = run({})
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)


CASES_OPS_3D = [
    ((64, 64, 64), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2, fcycle=True)),
    ((128, 128, 128), dict(precision="mixed", stop="residual", outer="fcg", inner_cycles=2, fcycle=True)),
    ((64, 64, 64), dict(stop="residual", outer="fcg")),
    ((64, 32, 128), dict(precision="mixed", fixed=True, max_iters_outer=5, gamma=2)),
    ((64, 64, 64), dict(fixed=True, max_iters_outer=4, nu1=2, nu2=1)),
    ((64, 64, 64), dict(precision="mixed", fixed=True, max_iters_outer=4, nu1=1, nu2=3)),
    ((64, 64, 64), dict(fixed=True, max_iters_outer=3, nu1=2, nu2=0)),
    ((64, 64, 64), dict(fixed=True, max_iters_outer=4, skip_pre=True, fcycle=True)),
    ((32, 64, 64), dict(fixed=True, max_iters_outer=3, fcycle=True, gamma=2)),
    ((64, 64, 64), dict()),
]


@pytest.mark.parametrize("shape,opts", CASES_OPS_3D, ids=lambda x: str(x))
def test_fused_operator_pairs_3d_equal_unfused(monkeypatch, shape, opts):
    """3D solves with the fused pairs on the levels of at most 2^19 points (smooth +
    restrict, prolong + smooth over tiles with halos; JMG_FUSEDOPS3D=1) and with the
    separate colour passes, tiled restriction and cell prolongation (the default): the same
    bits and counts, in FP64 and FP32 cycles, every cycle shape and sweep count."""
    grids = tuple(grid_1D(m) for m in shape)
    args = _problem(*shape, seed=11 + sum(shape))

    def run(env):
        monkeypatch.delenv("JMG_FUSEDOPS3D", raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        _engine.CACHE.plans.clear()
        _engine.CACHE.ws.clear()
        return solve_3d(*grids, *args, **opts)

    ref, c_ref = run({})
    got, c_got = run({"JMG_FUSEDOPS3D": "1"})
    assert int(c_got) == int(c_ref)
    assert torch.equal(got, ref)
