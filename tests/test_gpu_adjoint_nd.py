"""Hand-written adjoint of the fixed-mode 3D solve and of the 2D 9-point (D_xy) solve
against autograd and central differences.

The reference gets reverse mode from jax.vjp through its fixed loop (solver_2d.py:18-26,
461-463; solver_3d.py:468-470) and checks it with jax.test_util.check_grads
(tests/test_solver_2d.py:200-207). JAX cannot run here, so the checker is torch autograd
through float64 CPU restatements of the same fixed-mode solves (oracle/torch3d.py and
oracle/torch2d.py with D_xy, bit-identical in the forward to the pinned oracles):
gradients with respect to every input must agree to 1e-10 relative L2. The sizes put the
fine levels on the grid-wide kernels and the small levels on the single-block segments
(2048 padded points), and 3D 32^3 / 2D 128^2 also run a coarse level grid-wide. Central
differences (step 1e-6) on random directions check the same gradients independently.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import problems as P  # noqa: E402
from jsolver_gb300 import workloads as W  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d  # noqa: E402
from jsolver_gb300.solver_3d import solve_3d  # noqa: E402
from oracle.torch2d import Torch2D  # noqa: E402
from oracle.torch3d import Torch3D  # noqa: E402

DEV = torch.device("cuda", 0)
NAMES3 = ("phi0", "rhs", "lam", "D_xx", "D_yy", "D_zz")
NAMES9 = ("phi0", "rhs", "lam", "D_xx", "D_yy", "D_xy")


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def _problem3(mx, my, mz, seed):
    rng = np.random.default_rng(seed)
    shape = (mz + 3, my + 3, mx + 3)
    if mx == my == mz:
        p = W.random_3d(mx, seed=seed)
    else:
        p = dict(rhs=rng.standard_normal(shape), lam=rng.uniform(0, 10, shape),
                 **{k: np.exp(rng.standard_normal(shape)) for k in ("D_xx", "D_yy", "D_zz")})
    p["phi0"] = rng.standard_normal(shape) * 0.1  # a nonzero start exercises dL/dphi0
    return p, rng.standard_normal(shape)


def _problem9(mx, my, seed):
    rng = np.random.default_rng(seed)
    shape = (my + 3, mx + 3)
    D = [np.exp(0.5 * rng.standard_normal(shape)) for _ in range(2)]
    p = dict(phi0=rng.standard_normal(shape) * 0.1, rhs=rng.standard_normal(shape), lam=rng.uniform(0, 5, shape),
             D_xx=D[0], D_yy=D[1], D_xy=0.3 * np.minimum(D[0], D[1]) * rng.uniform(-1, 1, shape))
    return p, rng.standard_normal(shape)


def _gpu3(grids, p, w, **opts):
    ts = {k: torch.tensor(p[k], device=DEV, requires_grad=True) for k in NAMES3}
    phi, _ = solve_3d(*grids, *[ts[k] for k in NAMES3], fixed=True, **opts)
    loss = (phi * torch.tensor(w, device=DEV)).sum()
    loss.backward()
    return float(loss.detach()), {k: ts[k].grad.cpu().numpy() for k in NAMES3}


def _gpu9(grids, p, w, **opts):
    ts = {k: torch.tensor(p[k], device=DEV, requires_grad=True) for k in NAMES9}
    phi, _ = solve_2d(*grids, *[ts[k] for k in NAMES9[:5]], D_xy=ts["D_xy"], fixed=True, **opts)
    loss = (phi * torch.tensor(w, device=DEV)).sum()
    loss.backward()
    return float(loss.detach()), {k: ts[k].grad.cpu().numpy() for k in NAMES9}


def _ref3(grids, p, w, iters, **form):
    t = Torch3D(grids[0].mx, grids[1].mx, grids[2].mx, [g.idel for g in grids], **form)
    ts = {k: torch.tensor(p[k], requires_grad=True) for k in NAMES3}
    phi = t.solve_fixed(*[ts[k] for k in NAMES3], iters=iters)
    loss = (phi * torch.tensor(w)).sum()
    loss.backward()
    return float(loss.detach()), {k: ts[k].grad.numpy() for k in NAMES3}


def _ref9(grids, p, w, iters, **form):
    t = Torch2D(grids[0].mx, grids[1].mx, grids[0].idel, grids[1].idel, **form)
    ts = {k: torch.tensor(p[k], requires_grad=True) for k in NAMES9}
    phi = t.solve_fixed(*[ts[k] for k in NAMES9[:5]], iters=iters, Dxy=ts["D_xy"])
    loss = (phi * torch.tensor(w)).sum()
    loss.backward()
    return float(loss.detach()), {k: ts[k].grad.numpy() for k in NAMES9}


def _check(loss, g, rloss, rg, names):
    assert abs(loss - rloss) <= 1e-12 * abs(rloss), (loss, rloss)
    for k in names:
        assert _rel(g[k], rg[k]) < 1e-10, (k, _rel(g[k], rg[k]))


@pytest.mark.parametrize("ms,iters,form", [
    ((16, 16, 16), 3, {}), ((16, 32, 16), 2, {}), ((32, 16, 16), 2, {"gamma": 2}), ((16, 16, 16), 2, {"fcycle": True}),
    ((16, 16, 16), 3, {"nu1": 2, "nu2": 0}), ((16, 16, 16), 2, {"nu1": 0, "nu2": 2}), ((16, 16, 16), 3, {"skip_pre": True}),
    ((32, 32, 32), 2, {})], ids=["V", "V-aniso", "W", "F", "nu2-0", "nu1-0", "skip_pre", "V-32"])
def test_adjoint3d_matches_autograd(ms, iters, form):
    grids = tuple(grid_1D(m) for m in ms)
    p, w = _problem3(*ms, 3)
    loss, g = _gpu3(grids, p, w, max_iters_outer=iters, **form)
    rloss, rg = _ref3(grids, p, w, iters, **form)
    _check(loss, g, rloss, rg, NAMES3)


@pytest.mark.parametrize("ms,iters,form", [
    ((32, 32), 3, {}), ((64, 32), 2, {}), ((32, 32), 2, {"gamma": 2}), ((32, 32), 2, {"fcycle": True}),
    ((16, 16), 3, {"nu1": 2, "nu2": 0}), ((32, 32), 2, {"nu1": 0, "nu2": 2}), ((32, 32), 3, {"skip_pre": True}),
    ((128, 128), 2, {})], ids=["V", "V-aniso", "W", "F", "nu2-0", "nu1-0", "skip_pre", "V-128"])
def test_adjoint_dxy_matches_autograd(ms, iters, form):
    grids = tuple(grid_1D(m) for m in ms)
    p, w = _problem9(*ms, 4)
    loss, g = _gpu9(grids, p, w, max_iters_outer=iters, **form)
    rloss, rg = _ref9(grids, p, w, iters, **form)
    _check(loss, g, rloss, rg, NAMES9)


def test_adjoint_dxy_golden_problems(goldens):
    """Reverse mode on the reference's D_xy problems (7, 9, 10, 11 of
    tests/test_solver_2d.py:558-901) at 64^2, three fixed cycles from zero."""
    done = 0
    for r in goldens["tests_2d"]:
        if r["problem"] not in (7, 9, 10, 11) or tuple(r["res"]) != (64, 64):
            continue
        gx, gy, shape, _, rhs, lam, D = P.make_2d(r["problem"], 64, 64, grid_1D)
        rhs = W._zero_frame(rhs)  # problem 11 has a NaN on the frame, which no interior value reads
        lam = np.broadcast_to(lam, shape).copy() if np.ndim(lam) > 0 else np.full(shape, float(lam))
        # The torch restatement also evaluates the updates of the frame ring that do_BCs
        # discards; A_cc vanishes there in problems 7, 9 and 10, and its backward then
        # forms 0/0. lambda on the frame feeds no interior value (injection maps the frame
        # ring to the frame ring), so setting it to 1 changes neither phi nor any interior
        # gradient.
        ring = np.ones(shape, bool)
        ring[2:-2, 2:-2] = False
        lam[ring] = 1.0
        D = [np.broadcast_to(a, shape).copy() if np.ndim(a) > 0 else np.full(shape, float(a)) for a in D]
        p = dict(phi0=np.zeros(shape), rhs=rhs, lam=lam, D_xx=D[0], D_yy=D[1], D_xy=D[2])
        w = np.random.default_rng(r["problem"]).standard_normal(shape)
        loss, g = _gpu9((gx, gy), p, w, max_iters_outer=3)
        rloss, rg = _ref9((gx, gy), p, w, 3)
        _check(loss, g, rloss, rg, NAMES9)
        done += 1
    assert done == 4


def test_adjoint3d_scalar_coefficients():
    """Scalar lambda and D: the gradient is the sum over the array the scalar stands for."""
    grids = (grid_1D(16),) * 3
    p, w = _problem3(16, 16, 16, 5)
    ts = {k: torch.tensor(p[k], device=DEV, requires_grad=True) for k in ("phi0", "rhs")}
    sc = {k: torch.tensor(v, dtype=torch.float64, device=DEV, requires_grad=True)
          for k, v in (("lam", 2.0), ("D_xx", 1.5), ("D_yy", 0.7), ("D_zz", 1.1))}
    phi, _ = solve_3d(*grids, ts["phi0"], ts["rhs"], sc["lam"], sc["D_xx"], sc["D_yy"], sc["D_zz"], fixed=True,
                      max_iters_outer=2)
    (phi * torch.tensor(w, device=DEV)).sum().backward()
    q = dict(p, **{k: np.full(p["rhs"].shape, float(v)) for k, v in sc.items()})
    _, rg = _ref3(grids, q, w, 2)
    for k in ("lam", "D_xx", "D_yy", "D_zz"):
        assert abs(float(sc[k].grad) - rg[k].sum()) <= 1e-10 * np.abs(rg[k]).sum(), k
    assert _rel(ts["rhs"].grad.cpu().numpy(), rg["rhs"]) < 1e-10


@pytest.mark.parametrize("case", ["3d", "dxy"])
def test_adjoint_nd_central_differences(case):
    """18 random directions, central differences with step 1e-6 (relative to each input),
    measured against ||dL/dx|| ||v|| as in the 2D adjoint's check."""
    iters = 4
    if case == "3d":
        grids, names = (grid_1D(16),) * 3, NAMES3
        p, w = _problem3(16, 16, 16, 7)
        _, g = _gpu3(grids, p, w, max_iters_outer=iters)

        def solve(q):
            return solve_3d(*grids, *[torch.tensor(q[k], device=DEV) for k in names], fixed=True,
                            max_iters_outer=iters)[0]
    else:
        grids, names = (grid_1D(64),) * 2, NAMES9
        p, w = _problem9(64, 64, 7)
        _, g = _gpu9(grids, p, w, max_iters_outer=iters)

        def solve(q):
            return solve_2d(*grids, *[torch.tensor(q[k], device=DEV) for k in names[:5]],
                            D_xy=torch.tensor(q["D_xy"], device=DEV), fixed=True, max_iters_outer=iters)[0]
    wt = torch.tensor(w, device=DEV)
    rng = np.random.default_rng(11)
    h, worst = 1e-6, 0.0
    for d in range(18):
        k = names[d % len(names)]
        scale = np.abs(p[k]) + 1e-3 if k in ("lam", "D_xx", "D_yy", "D_zz", "D_xy") else 1.0
        v = rng.standard_normal(p[k].shape) * scale
        lp = float((solve(dict(p, **{k: p[k] + h * v})) * wt).sum())
        lm = float((solve(dict(p, **{k: p[k] - h * v})) * wt).sum())
        fd = (lp - lm) / (2 * h)
        ad = float(np.sum(g[k] * v))
        worst = max(worst, abs(fd - ad) / (np.linalg.norm(g[k]) * np.linalg.norm(v)))
    assert worst < 1e-6, worst


def test_adjoint_rejects_mixed_and_fcg():
    grids = (grid_1D(16),) * 3
    p, _ = _problem3(16, 16, 16, 1)
    ts = [torch.tensor(p[k], device=DEV, requires_grad=True) for k in NAMES3]
    for opts in ({"precision": "mixed"}, {"outer": "fcg"}):
        with pytest.raises(NotImplementedError, match="FP64 fixed-mode"):
            solve_3d(*grids, *ts, fixed=True, max_iters_outer=2, **opts)
