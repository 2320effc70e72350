"""D_xy (2D 9-point stencil) on the GPU against the oracle and the reference's goldens.

With D_xy and array D the reference adds the diagonal couplings A_ll, A_rl, A_lr, A_rr
(solver_2d.py:410-416), sweeps the four sub-lattices one after the other
(solver_2d.py:684-690) and prolongates the (even, even) points too (solver_2d.py:665).
Tolerances as in test_gpu_parity: fixed-count solves 1e-12 relative L2 against the NumPy
oracle (the C restatement has no 9-point stencil), golden counts exactly and RMSE within
the reference's own tolerance.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import problems as P  # noqa: E402
from jsolver_gb300 import _engine  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d, solve_2d_simple  # noqa: E402
from oracle import mg2d  # noqa: E402


def rel_l2(a, b):
    return float(np.linalg.norm((np.asarray(a) - b).ravel()) / max(np.linalg.norm(np.asarray(b).ravel()), 1e-300))


def test_golden_2d_dxy_problems(goldens):
    done = 0
    for r in goldens["tests_2d"]:
        if r["problem"] not in (7, 9, 10, 11):
            continue
        mx, my = r["res"]
        gx, gy, shape, pe, rhs, lam, D = P.make_2d(r["problem"], mx, my, grid_1D)
        if np.ndim(lam) > 0:
            lam = np.broadcast_to(lam, shape).copy()
        D = [np.broadcast_to(a, shape).copy() if np.ndim(a) > 0 else a for a in D]
        assert len(D) == 3
        phi, count = solve_2d_simple(gx, gy, np.zeros(shape), rhs, lam, D[0], D[1], D_xy=D[2])
        assert count == r["iterations"], (r["test"], count, r["iterations"])
        assert P.rmse(pe, phi) == pytest.approx(r["rmse"], abs=2e-15, rel=1e-9), r["test"]
        done += 1
    assert done >= 12


def _random_dxy(m, seed):
    rng = np.random.default_rng(seed)
    shape = (m + 3, m + 3)
    dxx = np.exp(0.5 * rng.standard_normal(shape))
    dyy = np.exp(0.5 * rng.standard_normal(shape))
    dxy = 0.3 * np.minimum(dxx, dyy) * rng.uniform(-1, 1, shape)
    lam = rng.uniform(0, 5, shape)
    rhs = rng.standard_normal(shape)
    phi0 = rng.standard_normal(shape) * 0.1
    return phi0, rhs, lam, dxx, dyy, dxy


FORMS = [{}, {"gamma": 2}, {"fcycle": True}, {"skip_pre": True}, {"nu1": 2, "nu2": 1}, {"nu1": 1, "nu2": 0},
         {"nu1": 0, "nu2": 2}]


@pytest.mark.parametrize("form", FORMS, ids=lambda f: ",".join(f"{k}={v}" for k, v in f.items()) or "V")
@pytest.mark.parametrize("mx,my", [(64, 64), (32, 64)])
def test_dxy_fixed_parity(form, mx, my):
    rng_seed = 5 + mx + my
    phi0, rhs, lam, dxx, dyy, dxy = _random_dxy(max(mx, my), rng_seed)
    sl = (slice(0, my + 3), slice(0, mx + 3))
    args = [a[sl] for a in (phi0, rhs, lam, dxx, dyy)]
    gx, gy = grid_1D(mx), grid_1D(my)
    phi, c = solve_2d(gx, gy, *args, D_xy=dxy[sl], fixed=True, max_iters_outer=5, **form)
    ref, rc = mg2d.solve_2d(gx, gy, *args, D_xy=dxy[sl], fixed=True, max_iters_outer=5, **form)
    assert c == rc == 5
    assert rel_l2(phi, ref) < 1e-12, rel_l2(phi, ref)


def test_dxy_operators_match_oracle():
    m = 64
    phi0, rhs, lam, dxx, dyy, dxy = _random_dxy(m, 3)
    mg2d._zero_frame(phi0)  # the operator entry points take phi with the solver's zero frame
    g = grid_1D(m)
    ops = _engine.OperatorSet((g, g), lam, (dxx, dyy), dxy)
    o = mg2d.Oracle2D(g, g)
    o.setup(phi0, rhs, lam, dxx, dyy, dxy)
    sw = ops.sweep(phi0, rhs, 0).cpu().numpy()
    ref = o.rbgs(phi0.copy(), rhs, 0)
    assert rel_l2(sw, ref) < 1e-13
    rc = ops.restrict(phi0, rhs, 0).cpu().numpy()
    assert rel_l2(rc, o.defect(phi0, rhs, 0)) < 1e-13
    pc = np.random.default_rng(1).standard_normal(o.shapes[1])
    mg2d._zero_frame(pc)
    pr = ops.prolong_add(phi0, pc, 0).cpu().numpy()
    assert rel_l2(pr, phi0 + o.prolongate(pc, 0)) < 1e-13
    res = ops.residual(phi0, rhs, 0).cpu().numpy()
    assert rel_l2(res, o.defect_field(phi0, rhs, 0)) < 1e-13


@pytest.mark.parametrize("precision,outer", [("fp64", "richardson"), ("mixed", "richardson"), ("mixed", "fcg"),
                                              ("fp64", "fcg")])
def test_dxy_residual_stop_forms(precision, outer):
    m = 128
    phi0, rhs, lam, dxx, dyy, dxy = _random_dxy(m, 8)
    g = grid_1D(m)
    o = mg2d.Oracle2D(g, g)
    o.setup(phi0, rhs, lam, dxx, dyy, dxy)
    phi, c = solve_2d(g, g, phi0, rhs, lam, dxx, dyy, D_xy=dxy, stop="residual", rtol=1e-10, precision=precision,
                      outer=outer)
    assert o.rel_residual(phi, rhs) <= 2e-10
