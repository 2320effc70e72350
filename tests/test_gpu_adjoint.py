"""Hand-written adjoint of the fixed-mode 2D solve against autograd and finite differences.

The reference checks reverse mode with jax.test_util.check_grads (tests/test_solver_2d.py:
200-207). JAX cannot run here, so the checker is torch autograd through a float64 CPU
restatement of the same fixed-mode solve (oracle/torch2d.py, bit-identical to the pinned
oracle): gradients with respect to phi0, rhs, lambda, D_xx and D_yy must agree to 1e-10
relative L2. Central finite differences (step 1e-6) on random directions check the same
gradients independently.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from jsolver_gb300 import workloads as W  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d  # noqa: E402
from oracle.torch2d import Torch2D  # noqa: E402

DEV = torch.device("cuda", 0)
NAMES = ("phi0", "rhs", "lam", "D_xx", "D_yy")


def _problem(mx, my, seed):
    rng = np.random.default_rng(seed)
    if mx == my:
        p = W.random_2d(mx, seed=seed)
    else:
        shape = (my + 3, mx + 3)
        p = dict(phi0=np.zeros(shape), rhs=rng.standard_normal(shape), lam=rng.uniform(0, 10, shape),
                 D_xx=np.exp(rng.standard_normal(shape)), D_yy=np.exp(rng.standard_normal(shape)))
    p["phi0"] = rng.standard_normal(p["rhs"].shape) * 0.1  # a nonzero start exercises dL/dphi0
    w = rng.standard_normal(p["rhs"].shape)
    return p, w


def _gpu_grads(gx, gy, p, w, **opts):
    ts = {k: torch.tensor(p[k], device=DEV, requires_grad=True) for k in NAMES}
    phi, _ = solve_2d(gx, gy, *[ts[k] for k in NAMES], fixed=True, **opts)
    loss = (phi * torch.tensor(w, device=DEV)).sum()
    loss.backward()
    return float(loss.detach()), {k: ts[k].grad.cpu().numpy() for k in NAMES}


def _ref_grads(gx, gy, p, w, iters, gamma=1, fcycle=False, nu1=1, nu2=1):
    t = Torch2D(gx.mx, gy.mx, gx.idel, gy.idel, gamma=gamma, fcycle=fcycle, nu1=nu1, nu2=nu2)
    ts = {k: torch.tensor(p[k], requires_grad=True) for k in NAMES}
    phi = t.solve_fixed(*[ts[k] for k in NAMES], iters=iters)
    loss = (phi * torch.tensor(w)).sum()
    loss.backward()
    return float(loss.detach()), {k: ts[k].grad.numpy() for k in NAMES}


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("mx,my,iters,form", [
    (32, 32, 4, {}), (32, 64, 3, {}), (32, 32, 3, {"gamma": 2}), (32, 32, 3, {"fcycle": True}),
    (16, 16, 5, {"nu1": 2, "nu2": 1}), (16, 16, 4, {"nu1": 1, "nu2": 0}), (16, 32, 2, {"nu1": 0, "nu2": 2})])
def test_adjoint_matches_autograd(mx, my, iters, form):
    gx, gy = grid_1D(mx), grid_1D(my)
    p, w = _problem(mx, my, 3)
    loss, g = _gpu_grads(gx, gy, p, w, max_iters_outer=iters, **form)
    rloss, rg = _ref_grads(gx, gy, p, w, iters, **form)
    assert abs(loss - rloss) <= 1e-12 * abs(rloss)
    for k in NAMES:
        assert _rel(g[k], rg[k]) < 1e-10, (k, _rel(g[k], rg[k]))


def test_adjoint_skip_pre_matches_autograd():
    gx = gy = grid_1D(32)
    p, w = _problem(32, 32, 5)
    loss, g = _gpu_grads(gx, gy, p, w, max_iters_outer=3, skip_pre=True)
    # skip_pre: one pre-smoothing before the loop, none at level 0 inside the cycles
    t = Torch2D(32, 32, gx.idel, gy.idel)
    ts = {k: torch.tensor(p[k], requires_grad=True) for k in NAMES}
    H = t.hierarchy(ts["lam"], ts["D_xx"], ts["D_yy"])
    phi = t.rbgs(ts["phi0"], ts["rhs"], H[0])
    for _ in range(3):
        phi = _cycle_skip(t, phi, ts["rhs"], H)
    (phi * torch.tensor(w)).sum().backward()
    for k in NAMES:
        assert _rel(g[k], ts[k].grad.numpy()) < 1e-10, k


def _cycle_skip(t, phi, rhs, H):
    from oracle.torch2d import _frame0
    phi = _frame0(phi)
    rc = t.defect(phi, rhs, H[0], 0)
    pc = torch.zeros(t.shapes[1], dtype=torch.float64)
    pc = t.cycle(pc, rc, H, False, 1)
    phi = phi + t.prolongate(pc, 0)
    return t.rbgs(phi, rhs, H[0])


def test_adjoint_central_differences():
    """32 random directions, central differences with step 1e-6 (relative to each input).

    The error is measured against ||dL/dx|| ||v||, the largest directional derivative the
    input x can have, so directions whose derivative nearly cancels do not inflate it."""
    m, iters = 64, 6
    gx = gy = grid_1D(m)
    p, w = _problem(m, m, 7)
    loss, g = _gpu_grads(gx, gy, p, w, max_iters_outer=iters)
    rng = np.random.default_rng(11)
    wt = torch.tensor(w, device=DEV)

    def L(q):
        phi, _ = solve_2d(gx, gy, *[torch.tensor(q[k], device=DEV) for k in NAMES], fixed=True,
                          max_iters_outer=iters)
        return float((phi * wt).sum())

    h = 1e-6
    worst = 0.0
    for d in range(32):
        k = NAMES[d % 5]
        v = rng.standard_normal(p[k].shape) * (np.abs(p[k]) + 1e-3 if k in ("lam", "D_xx", "D_yy") else 1.0)
        qp = dict(p)
        qm = dict(p)
        qp[k] = p[k] + h * v
        qm[k] = p[k] - h * v
        fd = (L(qp) - L(qm)) / (2 * h)
        ad = float(np.sum(g[k] * v))
        worst = max(worst, abs(fd - ad) / (np.linalg.norm(g[k]) * np.linalg.norm(v)))
    assert worst < 1e-6, worst


def test_dynamic_mode_is_not_reverse_differentiable():
    gx = gy = grid_1D(16)
    p, w = _problem(16, 16, 1)
    t = torch.tensor(p["rhs"], device=DEV, requires_grad=True)
    with pytest.raises(ValueError, match="fixed=True"):
        solve_2d(gx, gy, torch.tensor(p["phi0"], device=DEV), t, torch.tensor(p["lam"], device=DEV),
                 torch.tensor(p["D_xx"], device=DEV), torch.tensor(p["D_yy"], device=DEV))
