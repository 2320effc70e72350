"""Forward mode (JVP) of the solve against torch forward-mode AD and finite differences.

The reference gets forward-mode derivatives from jax.jvp through its solve and checks
them on every problem, through the dynamic loop (tests/test_solver_2d.py:173-176,
tests/test_solver_3d.py:208-211, the D_xy problems 7, 9, 10 and 11 included). JAX is
absent here, so the checker is torch.func.jvp through the float64 CPU restatements of
the same solve (oracle/torch2d.py, oracle/torch3d.py, bit-identical to the pinned NumPy
oracles), run for the cycle count of the primal (jax.jvp of lax.while_loop stops on the
primal's test and does not differentiate the count). Bars:
  * the tangent within 1e-10 relative L2 of torch forward mode;
  * the primal phi and the dynamic count equal to the plain solve's (same arithmetic);
  * central differences (step 1e-6) within 1e-6 relative L2.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import problems as P  # noqa: E402
from jsolver_gb300 import adjoint  # noqa: E402
from jsolver_gb300 import workloads as W  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d, solve_2d_simple  # noqa: E402
from jsolver_gb300.solver_3d import solve_3d  # noqa: E402
from oracle import mg2d, mg3d  # noqa: E402
from oracle.torch2d import Torch2D  # noqa: E402
from oracle.torch3d import Torch3D  # noqa: E402

DEV = torch.device("cuda", 0)


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def _problem(shape, ndim, seed, dxy=False):
    """Random primals (phi0, rhs, lam, D..., [D_xy]) and tangents of the same forms."""
    rng = np.random.default_rng(seed)
    D = [np.exp(0.5 * rng.standard_normal(shape)) for _ in range(ndim)]
    prim = [rng.standard_normal(shape) * 0.1, rng.standard_normal(shape), rng.uniform(0, 5, shape)] + D
    tang = [rng.standard_normal(shape), rng.standard_normal(shape), rng.standard_normal(shape)] + \
        [rng.standard_normal(shape) * d for d in D]
    if dxy:
        prim.append(0.3 * np.minimum(D[0], D[1]) * rng.uniform(-1, 1, shape))
        tang.append(0.1 * rng.standard_normal(shape) * np.minimum(D[0], D[1]))
    return prim, tang


def _dev(xs):  # (np.ascontiguousarray would turn 0-d scalars into shape (1,))
    return [torch.as_tensor(np.asarray(x), dtype=torch.float64, device=DEV).contiguous() for x in xs]


def _cpu(xs):
    return tuple(torch.as_tensor(np.asarray(x), dtype=torch.float64).contiguous() for x in xs)


def _torch_jvp(ndim, ms, grids, prim, tang, iters, form):
    kw = {k: form[k] for k in ("gamma", "fcycle", "nu1", "nu2", "skip_pre") if k in form}
    if ndim == 2:
        t = Torch2D(ms[0], ms[1], grids[0].idel, grids[1].idel, **kw)
        f = (lambda *a: t.solve_fixed(*a[:5], iters, a[5])) if len(prim) == 6 else \
            (lambda *a: t.solve_fixed(*a, iters=iters))
    else:
        t = Torch3D(ms[0], ms[1], ms[2], [g.idel for g in grids], **kw)

        def f(*a):
            return t.solve_fixed(*a, iters=iters)
    return torch.func.jvp(f, _cpu(prim), _cpu(tang))


CASES_2D = [((32, 32), 4, {}), ((32, 64), 3, {}), ((32, 32), 3, {"gamma": 2}), ((32, 32), 3, {"fcycle": True}),
            ((16, 16), 4, {"nu1": 2, "nu2": 0}), ((32, 32), 3, {"skip_pre": True})]


@pytest.mark.parametrize("ms,iters,form", CASES_2D, ids=lambda x: str(x))
def test_jvp_2d_fixed_matches_torch_forward_mode(ms, iters, form):
    grids = tuple(grid_1D(m) for m in ms)
    prim, tang = _problem((ms[1] + 3, ms[0] + 3), 2, 5)
    phi, dphi, c = adjoint.jvp(grids, _dev(prim), _dev(tang), fixed=True, max_iters_outer=iters, **form)
    ref, dref = _torch_jvp(2, ms, grids, prim, tang, iters, form)
    assert int(c) == iters
    assert _rel(phi.cpu().numpy(), ref.numpy()) < 1e-12
    assert _rel(dphi.cpu().numpy(), dref.numpy()) < 1e-10, _rel(dphi.cpu().numpy(), dref.numpy())


@pytest.mark.parametrize("form", [{}, {"gamma": 2}, {"fcycle": True}, {"skip_pre": True}],
                         ids=lambda f: ",".join(f"{k}={v}" for k, v in f.items()) or "V")
@pytest.mark.parametrize("dxy", [False, True], ids=["5pt", "9pt"])
def test_jvp_2d_dynamic_matches_torch_forward_mode(form, dxy):
    """The dynamic loop (distance stop): the count and phi are the plain solve's, the
    tangent is torch's forward mode through that many cycles."""
    ms = (32, 32)
    grids = (grid_1D(32), grid_1D(32))
    prim, tang = _problem((35, 35), 2, 7, dxy=dxy)
    phi, dphi, c = adjoint.jvp(grids, _dev(prim), _dev(tang), **form)
    kw = {"D_xy": prim[5]} if dxy else {}
    plain, pc = solve_2d(*grids, *prim[:5], **kw, **form)
    ref_o, rc = mg2d.solve_2d(*grids, *prim[:5], **kw, **form)
    assert int(c) == pc == rc
    np.testing.assert_array_equal(phi.cpu().numpy(), plain)
    ref, dref = _torch_jvp(2, ms, grids, prim, tang, int(c), form)
    assert _rel(phi.cpu().numpy(), ref.numpy()) < 1e-12
    assert _rel(dphi.cpu().numpy(), dref.numpy()) < 1e-10, _rel(dphi.cpu().numpy(), dref.numpy())


CASES_3D = [((16, 16, 16), {}), ((8, 16, 8), {"gamma": 2}), ((16, 16, 16), {"fcycle": True}),
            ((16, 16, 16), {"skip_pre": True}), ((16, 8, 16), {"nu1": 2, "nu2": 0})]


@pytest.mark.parametrize("ms,form", CASES_3D, ids=lambda x: str(x))
@pytest.mark.parametrize("fixed", [True, False], ids=["fixed", "dynamic"])
def test_jvp_3d_matches_torch_forward_mode(ms, form, fixed):
    grids = tuple(grid_1D(m) for m in ms)
    shape = (ms[2] + 3, ms[1] + 3, ms[0] + 3)
    prim, tang = _problem(shape, 3, 11)
    kw = dict(fixed=True, max_iters_outer=3) if fixed else {}
    phi, dphi, c = adjoint.jvp(grids, _dev(prim), _dev(tang), **kw, **form)
    plain, pc = solve_3d(*grids, *prim, **kw, **form)
    if not fixed:
        _, rc = mg3d.solve_3d(*grids, *prim, **form)
        assert int(c) == pc == rc
    np.testing.assert_array_equal(phi.cpu().numpy(), plain)
    ref, dref = _torch_jvp(3, ms, grids, prim, tang, int(c), form)
    assert _rel(phi.cpu().numpy(), ref.numpy()) < 1e-12
    assert _rel(dphi.cpu().numpy(), dref.numpy()) < 1e-10, _rel(dphi.cpu().numpy(), dref.numpy())


def test_jvp_dxy_golden_problems(goldens):
    """Forward mode through the dynamic solve on the reference's D_xy problems (the
    problems its forward-mode check covers, tests/test_solver_2d.py:558-901) at 64^2:
    the golden cycle count, and the tangent in random directions against torch."""
    done = 0
    for r in goldens["tests_2d"]:
        if r["problem"] not in (7, 9, 10, 11) or tuple(r["res"]) != (64, 64):
            continue
        gx, gy, shape, pe, rhs, lam, D = P.make_2d(r["problem"], 64, 64, grid_1D)
        rhs = W._zero_frame(rhs)  # problem 11 has a NaN on the frame, which no interior value reads
        lam = np.broadcast_to(lam, shape).copy() if np.ndim(lam) > 0 else np.full(shape, float(lam))
        D = [np.broadcast_to(a, shape).copy() if np.ndim(a) > 0 else np.full(shape, float(a)) for a in D]
        prim = [np.zeros(shape), rhs, lam, D[0], D[1], D[2]]
        rng = np.random.default_rng(r["problem"])
        tang = [rng.standard_normal(shape) * 0.01, rng.standard_normal(shape), rng.standard_normal(shape),
                rng.standard_normal(shape) * 0.1, rng.standard_normal(shape) * 0.1,
                rng.standard_normal(shape) * 0.01]
        phi, dphi, c = adjoint.jvp((gx, gy), _dev(prim), _dev(tang))
        assert int(c) == r["iterations"], (r["test"], int(c))
        assert P.rmse(pe, phi.cpu().numpy()) == pytest.approx(r["rmse"], abs=2e-15, rel=1e-9)
        ref, dref = _torch_jvp(2, (64, 64), (gx, gy), prim, tang, int(c), {})
        assert _rel(dphi.cpu().numpy(), dref.numpy()) < 1e-10, (r["test"], _rel(dphi.cpu().numpy(), dref.numpy()))
        done += 1
    assert done == 4


@pytest.mark.parametrize("ndim,dxy", [(2, False), (2, True), (3, False)])
def test_jvp_central_differences(ndim, dxy):
    """Tangent of the dynamic solve against central differences of the plain solve (the
    count is that of the primal; a step of 1e-6 does not change it here)."""
    if ndim == 2:
        grids, shape = (grid_1D(64),) * 2, (67, 67)
        solve = solve_2d
    else:
        grids, shape = (grid_1D(16),) * 3, (19, 19, 19)
        solve = solve_3d
    prim, tang = _problem(shape, ndim, 13, dxy=dxy)
    Pd, Td = _dev(prim), _dev(tang)
    phi, dphi, c = adjoint.jvp(grids, Pd, Td, epsilon=1e-10)

    def run(sign):
        x = [p + sign * 1e-6 * v for p, v in zip(Pd, Td)]
        kw = {"D_xy": x[5]} if dxy else {}
        out, cc = solve(*grids, *x[:3 + ndim], epsilon=1e-10, fixed=True, max_iters_outer=int(c), **kw)
        return out

    fd = (run(1) - run(-1)) / 2e-6
    assert _rel(dphi.cpu().numpy(), fd.cpu().numpy()) < 1e-6


def test_jvp_scalar_coefficients():
    m, iters = 32, 3
    g = grid_1D(m)
    rng = np.random.default_rng(2)
    shape = (m + 3, m + 3)
    s = lambda v: torch.tensor(v, dtype=torch.float64, device=DEV)  # noqa: E731
    Pd = [torch.tensor(rng.standard_normal(shape) * 0.1, device=DEV), torch.tensor(rng.standard_normal(shape), device=DEV),
          s(0.7), s(1.3), s(0.6)]
    Td = [torch.tensor(rng.standard_normal(shape), device=DEV), torch.tensor(rng.standard_normal(shape), device=DEV),
          s(0.3), s(-0.2), s(0.5)]
    phi, dphi = adjoint.jvp_2d_fixed((g, g), Pd, Td, fixed=True, max_iters_outer=iters)
    h = 1e-6
    plus, _ = solve_2d(g, g, *[p + h * v for p, v in zip(Pd, Td)], fixed=True, max_iters_outer=iters)
    minus, _ = solve_2d(g, g, *[p - h * v for p, v in zip(Pd, Td)], fixed=True, max_iters_outer=iters)
    assert _rel(dphi.cpu().numpy(), ((plus - minus) / (2 * h)).cpu().numpy()) < 1e-6
    # the same against torch forward mode through the restatement (scalars as constant arrays)
    ref, dref = _torch_jvp(2, (m, m), (g, g), [x.cpu().numpy() for x in Pd], [x.cpu().numpy() for x in Td], iters, {})
    assert _rel(dphi.cpu().numpy(), dref.numpy()) < 1e-10


def test_torch_func_jvp_through_solve():
    """torch.func.jvp through solve_2d / solve_3d (the reference's jax.jvp(solve, ...)):
    the library's forward-mode rule runs, and gives the same tangent as adjoint.jvp."""
    g = grid_1D(32)
    prim, tang = _problem((35, 35), 2, 3)
    Pd, Td = _dev(prim), _dev(tang)

    def f2(*a):
        return solve_2d(g, g, *a)[0]

    phi, dphi = torch.func.jvp(f2, tuple(Pd), tuple(Td))
    phi_r, dphi_r, _ = adjoint.jvp((g, g), Pd, Td)
    assert torch.equal(phi, phi_r) and torch.equal(dphi, dphi_r)
    g3 = grid_1D(8)
    prim3, tang3 = _problem((11, 11, 11), 3, 4)
    P3, T3 = _dev(prim3), _dev(tang3)
    phi3, dphi3 = torch.func.jvp(lambda *a: solve_3d(g3, g3, g3, *a, fixed=True, max_iters_outer=3)[0], tuple(P3),
                                 tuple(T3))
    phi3_r, dphi3_r, _ = adjoint.jvp((g3,) * 3, P3, T3, fixed=True, max_iters_outer=3)
    assert torch.equal(phi3, phi3_r) and torch.equal(dphi3, dphi3_r)
    # forward_ad dual tensors and solve_2d_simple (a wrapper) take the same rule
    import torch.autograd.forward_ad as fwAD
    with fwAD.dual_level():
        duals = [fwAD.make_dual(p, t) for p, t in zip(Pd, Td)]
        out, _ = solve_2d_simple(g, g, *duals)
        tangent = fwAD.unpack_dual(out).tangent
    assert torch.equal(tangent, dphi_r)


def test_jvp_rejects_other_forms():
    g = grid_1D(16)
    prim, tang = _problem((19, 19), 2, 1)
    with pytest.raises(ValueError, match="FP64 iteration"):
        adjoint.jvp((g, g), _dev(prim), _dev(tang), precision="mixed", fixed=True, max_iters_outer=2)
    with pytest.raises(ValueError, match="distance stop"):
        adjoint.jvp((g, g), _dev(prim), _dev(tang), stop="residual")
