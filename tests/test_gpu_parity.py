"""GPU parity: the CUDA solver (through the C ABI) against the oracle and the reference goldens.

Tolerances:
  * coefficient hierarchy: bit-exact (same operations in the same order);
  * one operator application (sweep, defect+restriction, prolongation): relative 1e-13
    (the GPU multiplies by 1/A_cc and fuses multiply-adds; the reference divides);
  * full solves: phi within 1e-12 relative L2 of the oracle at the same cycle count, the
    reference's golden iteration counts exactly, and the golden RMSE within the
    reference's own tolerance (pytest.approx rel 1e-9, abs 2e-15).
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import problems as P  # noqa: E402
from jsolver_gb300 import _engine, _lib  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import Solver_2D, solve_2d, solve_2d_simple  # noqa: E402
from jsolver_gb300.solver_3d import Solver_3D, solve_3d, solve_3d_simple  # noqa: E402
from jsolver_gb300 import workloads as W  # noqa: E402
from oracle import c_oracle, mg2d, mg3d  # noqa: E402

DEV = torch.device("cuda", 0)


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def t(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


def rand2d(mx, my, seed, scalar_D=False, scalar_lam=False):
    rng = np.random.default_rng(seed)
    shape = (my + 3, mx + 3)
    D = (1.0, 0.25) if scalar_D else tuple(np.exp(rng.standard_normal(shape)) for _ in range(2))
    lam = 0.5 if scalar_lam else rng.uniform(0, 5, shape)
    return shape, D, lam, rng.standard_normal(shape), rng.standard_normal(shape)


def rand3d(mx, my, mz, seed, scalar_D=False, scalar_lam=False):
    rng = np.random.default_rng(seed)
    shape = (mz + 3, my + 3, mx + 3)
    D = (1.0, 0.5, 2.0) if scalar_D else tuple(np.exp(rng.standard_normal(shape)) for _ in range(3))
    lam = 0.5 if scalar_lam else rng.uniform(0, 5, shape)
    return shape, D, lam, rng.standard_normal(shape), rng.standard_normal(shape)


# ---------------------------------------------------------------------------------------
# operators
# ---------------------------------------------------------------------------------------

@pytest.mark.parametrize("mx,my,scalar_D,scalar_lam", [(32, 64, False, False), (16, 16, True, False),
                                                       (64, 32, False, True), (8, 8, True, True)])
def test_hierarchy_2d_bit_exact(mx, my, scalar_D, scalar_lam):
    shape, D, lam, _, _ = rand2d(mx, my, 1, scalar_D, scalar_lam)
    gx, gy = grid_1D(mx), grid_1D(my)
    s = Solver_2D(gx, gy).setup(lam if scalar_lam else t(lam), *(D if scalar_D else map(t, D)))
    o = mg2d.Oracle2D(gx, gy)
    h = o.setup(np.zeros(shape), np.zeros(shape), lam, *D)
    for lvl in range(o.levels - 1):
        st = h.stencil(lvl)
        acc = s._ops.coeff(lvl, 0).cpu().numpy()
        wx = s._ops.coeff(lvl, 1).cpu().numpy()
        wy = s._ops.coeff(lvl, 2).cpu().numpy()
        np.testing.assert_array_equal(acc[2:-2, 2:-2], st["cc"][1:-1, 1:-1])
        np.testing.assert_array_equal(wx[2:-2, 2:-2], st["rc"][1:-1, 1:-1])
        np.testing.assert_array_equal(wx[2:-2, 1:-3], st["lc"][1:-1, 1:-1])
        np.testing.assert_array_equal(wy[2:-2, 2:-2], st["cr"][1:-1, 1:-1])
        np.testing.assert_array_equal(wy[1:-3, 2:-2], st["cl"][1:-1, 1:-1])


@pytest.mark.parametrize("mx,my,mz,scalar_D", [(16, 32, 16, False), (16, 16, 16, True), (32, 16, 8, False)])
def test_hierarchy_3d_bit_exact(mx, my, mz, scalar_D):
    shape, D, lam, _, _ = rand3d(mx, my, mz, 2, scalar_D)
    gs = (grid_1D(mx), grid_1D(my), grid_1D(mz))
    s = Solver_3D(*gs).setup(t(lam), *(D if scalar_D else map(t, D)))
    o = mg3d.Oracle3D(*gs)
    h = o.setup(np.zeros(shape), np.zeros(shape), lam, *D)
    i = (slice(2, -2),) * 3
    for lvl in range(o.levels - 1):
        st = h.stencil(lvl)
        acc, wx, wy, wz = (s._ops.coeff(lvl, w).cpu().numpy() for w in range(4))
        inner = (slice(1, -1),) * 3
        np.testing.assert_array_equal(acc[i], st["ccc"][inner])
        np.testing.assert_array_equal(wx[i], st["rcc"][inner])
        np.testing.assert_array_equal(wx[2:-2, 2:-2, 1:-3], st["lcc"][inner])
        np.testing.assert_array_equal(wy[i], st["crc"][inner])
        np.testing.assert_array_equal(wy[2:-2, 1:-3, 2:-2], st["clc"][inner])
        np.testing.assert_array_equal(wz[i], st["ccr"][inner])
        np.testing.assert_array_equal(wz[1:-3, 2:-2, 2:-2], st["ccl"][inner])


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("nu2", [1, 0])
def test_operators_match_oracle(dim, nu2):
    if dim == 2:
        shape, D, lam, phi, rhs = rand2d(32, 64, 3)
        gs = (grid_1D(32), grid_1D(64))
        s = Solver_2D(*gs, nu2=nu2).setup(t(lam), *map(t, D))
        o = mg2d.Oracle2D(*gs, nu2=nu2)
    else:
        shape, D, lam, phi, rhs = rand3d(16, 32, 16, 3)
        gs = (grid_1D(16), grid_1D(32), grid_1D(16))
        s = Solver_3D(*gs, nu2=nu2).setup(t(lam), *map(t, D))
        o = mg3d.Oracle3D(*gs, nu2=nu2)
    o.setup(np.zeros(shape), np.zeros(shape), lam, *D)
    for lvl in range(o.levels - 1):
        shp = o.shapes[lvl]
        rng = np.random.default_rng(lvl)
        ph = o.rbgs(rng.standard_normal(shp), rng.standard_normal(shp), lvl)  # zero frame, smoothed
        rh = rng.standard_normal(shp)
        # sweep
        ref = o.rbgs(ph.copy(), rh, lvl)
        got = s.red_black_gauss_seidel(t(ph), t(rh), lvl).cpu().numpy()
        assert rel_l2(got, ref) < 1e-13, (lvl, rel_l2(got, ref))
        if lvl + 1 < o.levels - 1:
            # defect + restriction
            ref = o.defect(ph, rh, lvl)
            got = s.defect(t(ph), t(rh), lvl).cpu().numpy()
            assert rel_l2(got, ref) < 1e-13, (lvl, rel_l2(got, ref))
            # prolongation
            pc = o.rbgs(rng.standard_normal(o.shapes[lvl + 1]), rng.standard_normal(o.shapes[lvl + 1]), lvl + 1)
            ref = o.prolongate(pc, lvl)
            got = s.prolongate(t(pc), lvl).cpu().numpy()
            np.testing.assert_array_equal(got, ref)


# ---------------------------------------------------------------------------------------
# reference goldens through the GPU
# ---------------------------------------------------------------------------------------

def _golden_2d(goldens, skip_dxy=True):
    for r in goldens["tests_2d"]:
        if skip_dxy and r["problem"] in (7, 9, 10, 11):
            continue
        yield r


def test_golden_2d_all(goldens):
    for r in _golden_2d(goldens):
        mx, my = r["res"]
        gx, gy, shape, pe, rhs, lam, D = P.make_2d(r["problem"], mx, my, grid_1D)
        if np.ndim(lam) > 0:
            lam = np.broadcast_to(lam, shape).copy()
        D = [np.broadcast_to(a, shape).copy() if np.ndim(a) > 0 else a for a in D]
        phi, count = solve_2d_simple(gx, gy, np.zeros(shape), rhs, lam, D[0], D[1])
        assert count == r["iterations"], (r["test"], count)
        assert P.rmse(pe, phi) == pytest.approx(r["rmse"], abs=2e-15, rel=1e-9), r["test"]
        ref, rc, _ = c_oracle.solve((gx, gy), np.zeros(shape), rhs, lam, D[:2], fixed=True, max_iters_outer=count)
        assert rel_l2(phi, ref) < 1e-12, (r["test"], rel_l2(phi, ref))


def test_golden_3d_all(goldens):
    for r in goldens["tests_3d"]:
        mx, my, mz = r["res"]
        gx, gy, gz, shape, pe, rhs, lam, D = P.make_3d(r["problem"], mx, my, mz, grid_1D)
        phi, count = solve_3d_simple(gx, gy, gz, np.zeros(shape), rhs, lam, *D)
        assert count == r["iterations"], (r["test"], count)
        assert P.rmse(pe, phi) == pytest.approx(r["rmse"], abs=2e-15, rel=1e-9), r["test"]
        ref, rc, _ = c_oracle.solve((gx, gy, gz), np.zeros(shape), rhs, lam, D, fixed=True, max_iters_outer=count)
        assert rel_l2(phi, ref) < 1e-12, (r["test"], rel_l2(phi, ref))


def test_golden_2d_test1_extras(goldens):
    """W, F, fixed and fixed-F checks of reference test1 (test_solver_2d.py:177-198)."""
    ex = goldens["test1_extras_2d"]
    gx, gy, shape, pe, rhs, lam, D = P.make_2d(1, 128, 128, grid_1D)
    phi, it = solve_2d(gx, gy, np.zeros(shape), rhs, lam, *D, fcycle=True)
    assert it <= ex["fcycle"]["max_iterations"]
    assert P.rmse(pe, phi) == pytest.approx(ex["fcycle"]["rmse"], rel=1e-9)
    phi, it = solve_2d(gx, gy, np.zeros(shape), rhs, lam, *D, gamma=2)
    assert it <= ex["wcycle"]["max_iterations"]
    assert P.rmse(pe, phi) == pytest.approx(ex["wcycle"]["rmse"], rel=1e-9)
    from jsolver_gb300.solver_2d import solve_2d_fixed_fcycle_simple, solve_2d_fixed_simple
    phi, it = solve_2d_fixed_simple(gx, gy, 13, np.zeros(shape), rhs, lam, *D)
    assert it == 13
    assert P.rmse(pe, phi) == pytest.approx(ex["fixed13"]["rmse"], abs=2e-15, rel=1e-9)
    phi, it = solve_2d_fixed_fcycle_simple(gx, gy, 13, np.zeros(shape), rhs, lam, *D)
    assert it == 13
    assert P.rmse(pe, phi) == pytest.approx(ex["fixed13_f"]["rmse"], rel=1e-9)


BENCH_MODES = {"reference_v": {}, "reference_vskip": {"skip_pre": True}, "reference_f": {"fcycle": True},
               "reference_fskip": {"fcycle": True, "skip_pre": True}, "reference_w": {"gamma": 2}}
# two benchmark-dictionary entries the oracle is not held to: (reference_v, 4, 64),
# whose RMSE contradicts the reference's own test4_64, and (reference_fskip, 9, 64), a
# D_xy problem one cycle off at the 1e-12 threshold (test_oracle_goldens.py)
KNOWN_BAD = {("reference_v", 4, 64), ("reference_fskip", 9, 64)}


@pytest.mark.parametrize("mode", sorted(BENCH_MODES))
def test_golden_benchmark_dicts(goldens, mode):
    for r in goldens["benchmark_2d"][mode]:
        if r["problem"] in (7, 9, 10, 11) or r["res"] > 256 or r["iterations"] > 2000:
            continue
        if (mode, r["problem"], r["res"]) in KNOWN_BAD:
            continue
        m = r["res"]
        gx, gy, shape, pe, rhs, lam, D = P.make_2d(r["problem"], m, m, grid_1D)
        if np.ndim(lam) > 0:
            lam = np.broadcast_to(lam, shape).copy()
        D = [np.broadcast_to(a, shape).copy() if np.ndim(a) > 0 else a for a in D]
        phi, count = solve_2d(gx, gy, np.zeros(shape), rhs, lam, D[0], D[1], **BENCH_MODES[mode])
        assert count == r["iterations"], (mode, r["problem"], m, count)
        if r["rmse"] is not None:
            assert P.rmse(pe, phi) == pytest.approx(r["rmse"], rel=1e-9), (mode, r["problem"], m)


# ---------------------------------------------------------------------------------------
# random coefficients, all cycle forms, fixed count parity at 1e-12
# ---------------------------------------------------------------------------------------

FORMS = [{}, {"gamma": 2}, {"fcycle": True}, {"skip_pre": True}, {"fcycle": True, "gamma": 2},
         {"nu1": 2, "nu2": 1}, {"nu1": 1, "nu2": 0}, {"nu1": 0, "nu2": 2}, {"gamma": 2, "skip_pre": True}]


@pytest.mark.parametrize("form", FORMS, ids=lambda f: ",".join(f"{k}={v}" for k, v in f.items()) or "V")
def test_random_2d_fixed_parity(form):
    p = W.random_2d(256, seed=7)
    g = grid_1D(256)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    phi, c = solve_2d(g, g, *args, fixed=True, max_iters_outer=8, **form)
    ref, _, _ = c_oracle.solve((g, g), args[0], args[1], args[2], args[3:], fixed=True, max_iters_outer=8, **form)
    assert c == 8
    assert rel_l2(phi, ref) < 1e-12, rel_l2(phi, ref)


@pytest.mark.parametrize("form", FORMS[:6], ids=lambda f: ",".join(f"{k}={v}" for k, v in f.items()) or "V")
def test_random_3d_fixed_parity(form):
    p = W.random_3d(32, seed=7)
    g = grid_1D(32)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
    phi, c = solve_3d(g, g, g, *args, fixed=True, max_iters_outer=6, **form)
    ref, _, _ = c_oracle.solve((g, g, g), args[0], args[1], args[2], args[3:], fixed=True, max_iters_outer=6, **form)
    assert rel_l2(phi, ref) < 1e-12, rel_l2(phi, ref)


def test_random_2d_dynamic_count_matches_oracle():
    p = W.random_2d(128, seed=11)
    g = grid_1D(128)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    phi, c = solve_2d(g, g, *args)
    ref, rc, _ = c_oracle.solve((g, g), args[0], args[1], args[2], args[3:])
    assert c == rc
    assert rel_l2(phi, ref) < 1e-12


def test_residual_stop_matches_oracle():
    p = W.random_2d(256, seed=5)
    g = grid_1D(256)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    phi, c = solve_2d(g, g, *args, stop="residual", rtol=1e-10)
    ref, rc, rr = c_oracle.solve((g, g), args[0], args[1], args[2], args[3:], stop="residual", rtol=1e-10)
    assert c == rc
    assert rr <= 1e-10
    o = mg2d.Oracle2D(g, g)
    o.setup(*args)
    assert o.rel_residual(phi, p["rhs"]) <= 1e-10


# ---------------------------------------------------------------------------------------
# edge cases
# ---------------------------------------------------------------------------------------

def test_zero_iterations_returns_input():
    shape, D, lam, phi, rhs = rand2d(16, 16, 4)
    g = grid_1D(16)
    out, c = solve_2d(g, g, phi, rhs, lam, *D, max_iters_outer=0)
    assert c == 0
    np.testing.assert_array_equal(out, phi)
    out, c = solve_2d(g, g, phi, rhs, lam, *D, fixed=True, max_iters_outer=0)
    assert c == 0
    np.testing.assert_array_equal(out, phi)


def test_nonzero_initial_frame_distance():
    """The first distance sees phi0's frame (solver_2d.py:471 copies phi before do_BCs)."""
    shape, D, lam, phi, rhs = rand2d(32, 32, 5)
    g = grid_1D(32)
    phi0 = phi * 1e3
    for eps in (1e-12, 1e-3):
        out, c = solve_2d(g, g, phi0, rhs, lam, *D, epsilon=eps)
        ref, rc = mg2d.solve_2d(g, g, phi0, rhs, lam, *D, epsilon=eps)
        assert c == rc
        assert rel_l2(out, ref) < 1e-12


def test_nan_ends_dynamic_loop():
    shape, D, lam, phi, rhs = rand2d(16, 16, 6)
    g = grid_1D(16)
    rhs = rhs.copy()
    rhs[5, 7] = np.nan
    out, c = solve_2d(g, g, np.zeros(shape), rhs, lam, *D)
    ref, rc = mg2d.solve_2d(g, g, np.zeros(shape), rhs, lam, *D)
    assert c == rc == 1
    assert np.isnan(out).sum() == np.isnan(ref).sum() > 0


def test_nan_in_frame_is_ignored():
    """rhs NaN on the frame (problem 11 has one at (1,1)) never reaches the interior."""
    shape, D, lam, phi, rhs = rand2d(16, 16, 8)
    g = grid_1D(16)
    rhs = rhs.copy()
    rhs[1, 1] = np.nan
    rhs[0, 5] = np.inf
    out, c = solve_2d(g, g, np.zeros(shape), rhs, lam, *D)
    ref, rc = mg2d.solve_2d(g, g, np.zeros(shape), rhs, lam, *D)
    assert c == rc and np.isfinite(out).all()
    assert rel_l2(out, ref) < 1e-12


def test_smallest_grids():
    for m in (2, 4, 8):
        shape, D, lam, phi, rhs = rand2d(m, m, m)
        g = grid_1D(m)
        out, c = solve_2d(g, g, np.zeros(shape), rhs, lam, *D)
        ref, rc = mg2d.solve_2d(g, g, np.zeros(shape), rhs, lam, *D)
        assert c == rc and rel_l2(out, ref) < 1e-12
    shape, D, lam, phi, rhs = rand3d(4, 8, 4, 1)
    gs = (grid_1D(4), grid_1D(8), grid_1D(4))
    out, c = solve_3d(*gs, np.zeros(shape), rhs, lam, *D)
    ref, rc = mg3d.solve_3d(*gs, np.zeros(shape), rhs, lam, *D)
    assert c == rc and rel_l2(out, ref) < 1e-12


def test_torch_inputs_stay_on_device():
    shape, D, lam, phi, rhs = rand2d(64, 64, 9)
    g = grid_1D(64)
    out, c = solve_2d(g, g, t(np.zeros(shape)), t(rhs), t(lam), t(D[0]), t(D[1]))
    assert out.is_cuda and isinstance(c, torch.Tensor) and c.is_cuda and c.dtype == torch.int64
    ref, rc = mg2d.solve_2d(g, g, np.zeros(shape), rhs, lam, *D)
    assert int(c.item()) == rc and rel_l2(out.cpu().numpy(), ref) < 1e-12
    out, c = solve_2d(g, g, t(np.zeros(shape)), t(rhs), t(lam), t(D[0]), t(D[1]), fixed=True, max_iters_outer=3)
    assert c == 3


def test_mixed_precision_reaches_rtol():
    p = W.random_2d(256, seed=3)
    g = grid_1D(256)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    phi64, c64 = solve_2d(g, g, *args, stop="residual", rtol=1e-10)
    phim, cm = solve_2d(g, g, *args, stop="residual", rtol=1e-10, precision="mixed")
    o = mg2d.Oracle2D(g, g)
    o.setup(*args)
    assert o.rel_residual(phim, p["rhs"]) <= 1e-10
    # both meet the residual tolerance; their difference is bounded by the operator's
    # conditioning times 1e-10 and is far below the discretisation error
    assert rel_l2(phim, phi64) < 1e-6
    assert rel_l2(phim, p["phi_exact"]) < 1e-6
    assert cm <= c64 + 5


def test_oneshot_c_abi():
    """jmg_solve2d_f64 called directly through ctypes with raw device pointers."""
    lib = _lib.load()
    shape, D, lam, phi, rhs = rand2d(64, 32, 10)
    gx, gy = grid_1D(64), grid_1D(32)
    grid = _engine.make_grid((gx, gy))
    cfg = _engine.make_config()
    plan = _lib.Plan(grid, cfg)
    ws = torch.empty(plan.workspace_bytes, dtype=torch.uint8, device=DEV)
    d = [t(x) for x in (np.zeros(shape), rhs, lam, D[0], D[1])]
    out = torch.empty_like(d[0])
    cnt = torch.zeros((), dtype=torch.int64, device=DEV)
    co = _lib.JmgCoeffs()
    co.lam = d[2].data_ptr()
    co.D[0], co.D[1] = d[3].data_ptr(), d[4].data_ptr()
    vp = ctypes.c_void_p
    rc = lib.jmg_solve2d_f64(ctypes.byref(grid), ctypes.byref(cfg), vp(d[0].data_ptr()), vp(d[1].data_ptr()),
                             ctypes.byref(co), vp(out.data_ptr()), vp(cnt.data_ptr()), vp(ws.data_ptr()),
                             ctypes.c_size_t(ws.numel()), vp(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc)
    ref, rcount = mg2d.solve_2d(gx, gy, np.zeros(shape), rhs, lam, *D)
    assert int(cnt.item()) == rcount and rel_l2(out.cpu().numpy(), ref) < 1e-12
    # too small a workspace is an error, not a fault
    rc = lib.jmg_solve2d_f64(ctypes.byref(grid), ctypes.byref(cfg), vp(d[0].data_ptr()), vp(d[1].data_ptr()),
                             ctypes.byref(co), vp(out.data_ptr()), vp(cnt.data_ptr()), vp(ws.data_ptr()),
                             ctypes.c_size_t(16), vp(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.JMG_ERR_WORKSPACE


def test_do_bcs_device():
    from jsolver_gb300.boundary_handler_2d import do_BCs as bc2
    from jsolver_gb300.boundary_handler_3d import do_BCs as bc3
    a = torch.ones((131, 131), dtype=torch.float64, device=DEV)
    np.testing.assert_array_equal(bc2(a).cpu().numpy(), mg2d.do_bcs(np.ones((131, 131))))
    b = torch.ones((11, 19, 7), dtype=torch.float64, device=DEV)
    np.testing.assert_array_equal(bc3(b).cpu().numpy(), mg3d.do_bcs(np.ones((11, 19, 7))))


def test_mixed_precision_3d_reaches_rtol():
    p = W.random_3d(32, seed=4)
    g = grid_1D(32)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
    phi64, c64 = solve_3d(g, g, g, *args, stop="residual", rtol=1e-10, fcycle=True)
    phim, cm = solve_3d(g, g, g, *args, stop="residual", rtol=1e-10, fcycle=True, precision="mixed")
    o = mg3d.Oracle3D(g, g, g)
    o.setup(*args)
    assert o.rel_residual(phim, p["rhs"]) <= 1e-10
    assert rel_l2(phim, phi64) < 1e-6
    assert cm <= c64 + 5


@pytest.mark.parametrize("dim", [2, 3])
def test_mixed_precision_fixed_and_distance_modes(dim):
    """The unfused refinement path (fixed count, distance stop) also converges to the FP64 answer."""
    if dim == 2:
        p = W.random_2d(64, seed=6)
        gs = (grid_1D(64),) * 2
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
        solve = solve_2d
    else:
        p = W.random_3d(16, seed=6)
        gs = (grid_1D(16),) * 3
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
        solve = solve_3d
    ref, _ = solve(*gs, *args, stop="residual", rtol=1e-11)
    phim, cm = solve(*gs, *args, precision="mixed", epsilon=1e-13)
    assert rel_l2(phim, ref) < 1e-7
    phif, cf = solve(*gs, *args, precision="mixed", fixed=True, max_iters_outer=cm)
    assert cf == cm and rel_l2(phif, phim) < 1e-12


CLUSTER_CASES = [(2, 64, {}), (2, 256, {}), (2, 256, {"gamma": 2}), (2, 256, {"fcycle": True}),
                 (2, 128, {"skip_pre": True}), (2, 128, {"nu1": 2, "nu2": 0}), (2, 128, {"nu1": 0, "nu2": 2}),
                 (2, 512, {"precision": "mixed"}), (3, 32, {"fcycle": True}), (3, 64, {}),
                 (3, 32, {"gamma": 2, "precision": "mixed"})]


@pytest.mark.parametrize("dim,m,form", CLUSTER_CASES,
                         ids=lambda x: ",".join(f"{k}={v}" for k, v in x.items()) if isinstance(x, dict) else str(x))
def test_cluster_coarse_cycle_matches_single_block(dim, m, form, monkeypatch):
    """The coarse levels on a thread-block cluster (JMG_COARSE=cluster: rows spread over
    the CTAs' shared memory) against the default single-block global-memory kernel: the
    same point arithmetic, so the same phi to rounding and the same cycle count."""
    g = grid_1D(m)
    if dim == 2:
        p = W.random_2d(m, seed=21)
        grids, fn = (g, g), solve_2d
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    else:
        p = W.random_3d(m, seed=21)
        grids, fn = (g, g, g), solve_3d
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
    kw = dict(form)
    if kw.get("precision") == "mixed":
        kw.update(stop="residual", rtol=1e-9)
    else:
        kw.update(fixed=True, max_iters_outer=5)
    phi_b, c_b = fn(*grids, *args, **kw)
    monkeypatch.setenv("JMG_COARSE", "cluster")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_c, c_c = fn(*grids, *args, **kw)
    assert int(c_c) == int(c_b)
    assert rel_l2(phi_c, phi_b) < 1e-13, rel_l2(phi_c, phi_b)


@pytest.mark.parametrize("dim,m,precision,form", [(2, 256, "fp64", {}), (2, 256, "mixed", {}), (2, 64, "fp64", {}),
                                                  (2, 128, "mixed", {"gamma": 2}), (3, 32, "fp64", {"fcycle": True}),
                                                  (3, 32, "mixed", {})])
def test_fcg_outer_reaches_rtol(dim, m, precision, form):
    """The cycle as the preconditioner of flexible CG (outer='fcg'): the true relative
    residual (oracle, FP64 on the CPU) meets the tolerance up to the recurrence's drift,
    in fewer cycles than the reference's stationary iteration, and the solution agrees
    with the FP64 stationary one to the accuracy the tolerance allows."""
    g = grid_1D(m)
    if dim == 2:
        p = W.random_2d(m, seed=9)
        grids, fn = (g, g), solve_2d
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
        o = mg2d.Oracle2D(g, g)
    else:
        p = W.random_3d(m, seed=9)
        grids, fn = (g, g, g), solve_3d
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
        o = mg3d.Oracle3D(g, g, g)
    o.setup(*args)
    ref, c_ref = fn(*grids, *args, stop="residual", rtol=1e-10, **form)
    phi, c = fn(*grids, *args, stop="residual", rtol=1e-10, precision=precision, outer="fcg", **form)
    rr = o.rel_residual(phi, p["rhs"])
    assert rr <= 2e-10, rr
    assert c < c_ref, (c, c_ref)
    assert rel_l2(phi, ref) < 1e-6


def test_fcg_outer_fixed_count_and_errors():
    g = grid_1D(64)
    p = W.random_2d(64, seed=2)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    phi, c = solve_2d(g, g, *args, fixed=True, max_iters_outer=7, outer="fcg")
    assert c == 7 and np.all(np.isfinite(phi))
    with pytest.raises(ValueError, match="fcg"):
        solve_2d(g, g, *args, outer="fcg")  # the distance stop measures a stationary iteration


@pytest.mark.parametrize("m,form", [(1024, {}), (256, {"gamma": 2}), (128, {"fcycle": True}), (64, {"skip_pre": True}),
                                    (512, {"outer": "fcg"})])
def test_mixed_coarse_from_shared_memory_matches_global(m, form, monkeypatch):
    """FP32 2D coarse levels staged in shared memory (opt-in, JMG_COARSE32=smem) against
    the default recursion reading global memory: identical arithmetic, so the same cycle
    count and phi to rounding."""
    p = W.random_2d(m, seed=4)
    g = grid_1D(m)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    kw = dict(stop="residual", rtol=1e-10, precision="mixed", **form)
    phi_g, c_g = solve_2d(g, g, *args, **kw)
    monkeypatch.setenv("JMG_COARSE32", "smem")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_s, c_s = solve_2d(g, g, *args, **kw)
    assert int(c_s) == int(c_g)
    assert rel_l2(phi_s, phi_g) < 1e-13, rel_l2(phi_s, phi_g)


STAGED_CASES = [(2, 1024, {"precision": "mixed", "outer": "fcg", "inner_cycles": 2}), (2, 256, {}),
                (2, 256, {"gamma": 2}), (2, 256, {"fcycle": True}), (2, 128, {"skip_pre": True}),
                (2, 128, {"nu1": 2, "nu2": 0}), (2, 128, {"nu1": 0, "nu2": 2}), (2, 512, {"precision": "mixed"}),
                (2, 8, {}), (3, 32, {"fcycle": True}), (3, 64, {}), (3, 32, {"gamma": 2, "precision": "mixed"}),
                (3, 64, {"precision": "mixed", "outer": "fcg", "fcycle": True})]


@pytest.mark.parametrize("dim,m,form", STAGED_CASES,
                         ids=lambda x: ",".join(f"{k}={v}" for k, v in x.items()) if isinstance(x, dict) else str(x))
def test_staged_coarse_cycle_matches_global(dim, m, form, monkeypatch):
    """The coarse sub-cycle with its levels staged in shared memory by bulk copies (the
    default) against the global-memory single-block kernel (JMG_COARSE=global): the same
    per-point functions on the same values, so the same bits and cycle counts."""
    g = grid_1D(m)
    if dim == 2:
        p = W.random_2d(m, seed=23)
        grids, fn = (g, g), solve_2d
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    else:
        p = W.random_3d(m, seed=23)
        grids, fn = (g, g, g), solve_3d
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
    kw = dict(form)
    if kw.get("precision") == "mixed" or kw.get("outer") == "fcg":
        kw.update(stop="residual", rtol=1e-9)
    else:
        kw.update(fixed=True, max_iters_outer=5)
    monkeypatch.setenv("JMG_COARSE", "global")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_g, c_g = fn(*grids, *args, **kw)
    monkeypatch.delenv("JMG_COARSE")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_s, c_s = fn(*grids, *args, **kw)
    assert int(c_s) == int(c_g)
    np.testing.assert_array_equal(phi_s, phi_g)


def test_staged_coarse_cycle_with_dxy(monkeypatch):
    """The staged kernel with the four D_xy diagonal arrays per level."""
    rng = np.random.default_rng(3)
    m = 128
    shape = (m + 3, m + 3)
    dxx, dyy = np.exp(0.5 * rng.standard_normal(shape)), np.exp(0.5 * rng.standard_normal(shape))
    dxy = 0.3 * np.minimum(dxx, dyy) * rng.uniform(-1, 1, shape)
    args = (np.zeros(shape), rng.standard_normal(shape), rng.uniform(0, 5, shape), dxx, dyy)
    g = grid_1D(m)
    monkeypatch.setenv("JMG_COARSE", "global")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_g, c_g = solve_2d(g, g, *args, D_xy=dxy, fixed=True, max_iters_outer=4)
    monkeypatch.delenv("JMG_COARSE")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_s, c_s = solve_2d(g, g, *args, D_xy=dxy, fixed=True, max_iters_outer=4)
    np.testing.assert_array_equal(phi_s, phi_g)
    ref, _ = mg2d.solve_2d(g, g, *args, D_xy=dxy, fixed=True, max_iters_outer=4)
    assert rel_l2(phi_s, ref) < 1e-12


OPS_CASES = [(2, 256, {}), (2, 256, {"gamma": 2}), (2, 256, {"fcycle": True}), (2, 128, {"fcycle": True, "gamma": 2}),
             (2, 8, {"skip_pre": True}), (2, 128, {"nu1": 2, "nu2": 0}), (2, 128, {"nu1": 0, "nu2": 2}),
             (2, 1024, {"precision": "mixed", "outer": "fcg", "inner_cycles": 2}), (3, 32, {"gamma": 2}),
             (3, 64, {"precision": "mixed", "outer": "fcg", "fcycle": True})]


@pytest.mark.parametrize("dim,m,form", OPS_CASES,
                         ids=lambda x: ",".join(f"{k}={v}" for k, v in x.items()) if isinstance(x, dict) else str(x))
@pytest.mark.parametrize("coarse", ["staged", "global"])
def test_coarse_op_list_matches_recursion(dim, m, form, coarse, monkeypatch):
    """The single-block coarse kernels walk a host-built list of the sub-cycle's operations;
    JMG_COARSE_OPS=0 makes them walk the recursion instead. Same operations in the same
    order, so the same bits and cycle counts, for every cycle shape and both kernels."""
    g = grid_1D(m)
    if dim == 2:
        p = W.random_2d(m, seed=29)
        grids, fn = (g, g), solve_2d
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    else:
        p = W.random_3d(m, seed=29)
        grids, fn = (g, g, g), solve_3d
        args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
    kw = dict(form)
    if kw.get("precision") == "mixed" or kw.get("outer") == "fcg":
        kw.update(stop="residual", rtol=1e-9)
    else:
        kw.update(fixed=True, max_iters_outer=4)
    if coarse == "global":
        monkeypatch.setenv("JMG_COARSE", "global")
    monkeypatch.setenv("JMG_COARSE_OPS", "0")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_r, c_r = fn(*grids, *args, **kw)
    monkeypatch.delenv("JMG_COARSE_OPS")
    monkeypatch.setattr(_engine, "CACHE", _engine._Cache())
    phi_l, c_l = fn(*grids, *args, **kw)
    assert int(c_r) == int(c_l)
    np.testing.assert_array_equal(phi_l, phi_r)
