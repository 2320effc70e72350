"""Forward mode (JVP) of the fixed-mode 2D solve against torch forward-mode AD and finite
differences.

The reference gets forward-mode derivatives from jax.jvp through its fixed loop. JAX is
absent here, so the checker is torch.func.jvp through the float64 CPU restatement of the
same fixed-mode solve (oracle/torch2d.py, bit-identical to the pinned oracle): the
tangent must agree to 1e-10 relative L2. Central differences (step 1e-6) check it
independently.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from jsolver_gb300 import adjoint  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d  # noqa: E402
from oracle.torch2d import Torch2D  # noqa: E402

DEV = torch.device("cuda", 0)


def _problem(mx, my, seed):
    rng = np.random.default_rng(seed)
    shape = (my + 3, mx + 3)
    prim = [rng.standard_normal(shape) * 0.1, rng.standard_normal(shape), rng.uniform(0, 5, shape),
            np.exp(rng.standard_normal(shape)), np.exp(rng.standard_normal(shape))]
    tang = [rng.standard_normal(shape), rng.standard_normal(shape), rng.standard_normal(shape),
            rng.standard_normal(shape) * prim[3], rng.standard_normal(shape) * prim[4]]
    return prim, tang


def _rel(a, b):
    return float(np.linalg.norm((np.asarray(a) - b).ravel()) / max(np.linalg.norm(np.asarray(b).ravel()), 1e-300))


@pytest.mark.parametrize("mx,my,iters,form", [(32, 32, 4, {}), (32, 64, 3, {}), (32, 32, 3, {"gamma": 2}),
                                              (32, 32, 3, {"fcycle": True}), (16, 16, 4, {"nu1": 2, "nu2": 0}),
                                              (32, 32, 3, {"skip_pre": True})])
def test_jvp_matches_torch_forward_mode(mx, my, iters, form):
    gx, gy = grid_1D(mx), grid_1D(my)
    prim, tang = _problem(mx, my, 5)
    phi, dphi = adjoint.jvp_2d_fixed((gx, gy), [torch.tensor(x, device=DEV) for x in prim],
                                     [torch.tensor(x, device=DEV) for x in tang], fixed=True,
                                     max_iters_outer=iters, **form)
    t = Torch2D(mx, my, gx.idel, gy.idel, **{k: v for k, v in form.items() if k != "skip_pre"})

    def f(*a):
        if form.get("skip_pre"):
            return _skip_pre_solve(t, gx, a, iters)
        return t.solve_fixed(*a, iters=iters)

    ref, dref = torch.func.jvp(f, tuple(torch.tensor(x) for x in prim), tuple(torch.tensor(x) for x in tang))
    assert _rel(phi.cpu().numpy(), ref.numpy()) < 1e-12
    assert _rel(dphi.cpu().numpy(), dref.numpy()) < 1e-10, _rel(dphi.cpu().numpy(), dref.numpy())


def _skip_pre_solve(t, g, a, iters):
    from oracle.torch2d import _frame0
    phi0, rhs, lam, dxx, dyy = a
    H = t.hierarchy(lam, dxx, dyy)
    phi = t.rbgs(phi0, rhs, H[0])
    for _ in range(iters):
        phi = _frame0(phi)
        rc = t.defect(phi, rhs, H[0], 0)
        pc = torch.zeros(t.shapes[1], dtype=torch.float64)
        pc = t.cycle(pc, rc, H, False, 1)
        phi = phi + t.prolongate(pc, 0)
        phi = t.rbgs(phi, rhs, H[0])
    return phi


def test_jvp_central_differences_and_primal():
    m, iters = 64, 5
    g = grid_1D(m)
    prim, tang = _problem(m, m, 9)
    P = [torch.tensor(x, device=DEV) for x in prim]
    Tn = [torch.tensor(x, device=DEV) for x in tang]
    phi, dphi = adjoint.jvp_2d_fixed((g, g), P, Tn, fixed=True, max_iters_outer=iters)
    plain, _ = solve_2d(g, g, *P, fixed=True, max_iters_outer=iters)
    # the primal of the dual solve is the solve itself (same arithmetic, other kernels)
    assert _rel(phi.cpu().numpy(), plain.cpu().numpy()) < 1e-13
    h = 1e-6
    plus, _ = solve_2d(g, g, *[p + h * v for p, v in zip(P, Tn)], fixed=True, max_iters_outer=iters)
    minus, _ = solve_2d(g, g, *[p - h * v for p, v in zip(P, Tn)], fixed=True, max_iters_outer=iters)
    fd = (plus - minus) / (2 * h)
    assert _rel(dphi.cpu().numpy(), fd.cpu().numpy()) < 1e-6


def test_jvp_scalar_coefficients():
    m, iters = 32, 3
    g = grid_1D(m)
    rng = np.random.default_rng(2)
    shape = (m + 3, m + 3)
    P = [torch.tensor(rng.standard_normal(shape) * 0.1, device=DEV), torch.tensor(rng.standard_normal(shape), device=DEV),
         torch.tensor(0.7, dtype=torch.float64, device=DEV), torch.tensor(1.3, dtype=torch.float64, device=DEV),
         torch.tensor(0.6, dtype=torch.float64, device=DEV)]
    Tn = [torch.tensor(rng.standard_normal(shape), device=DEV), torch.tensor(rng.standard_normal(shape), device=DEV),
          torch.tensor(0.3, dtype=torch.float64, device=DEV), torch.tensor(-0.2, dtype=torch.float64, device=DEV),
          torch.tensor(0.5, dtype=torch.float64, device=DEV)]
    phi, dphi = adjoint.jvp_2d_fixed((g, g), P, Tn, fixed=True, max_iters_outer=iters)
    h = 1e-6
    plus, _ = solve_2d(g, g, *[p + h * v for p, v in zip(P, Tn)], fixed=True, max_iters_outer=iters)
    minus, _ = solve_2d(g, g, *[p - h * v for p, v in zip(P, Tn)], fixed=True, max_iters_outer=iters)
    assert _rel(dphi.cpu().numpy(), ((plus - minus) / (2 * h)).cpu().numpy()) < 1e-6
