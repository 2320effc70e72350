"""Batched multi-solve (jmg_solve_batched): every problem's phi and count equal a single
solve of that problem, bit for bit, whatever the lane count and however the coefficients
are shared across the batch (the single solves are checked against the oracle in
test_gpu_parity.py); one case checks the batched results against the C oracle directly."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from jsolver_gb300 import workloads as W  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d, solve_2d_batched  # noqa: E402
from jsolver_gb300.solver_3d import solve_3d, solve_3d_batched  # noqa: E402

DEV = torch.device("cuda", 0)


def _stack(problems, key):
    return torch.from_numpy(np.stack([p[key] for p in problems])).to(DEV)


@pytest.mark.parametrize("lanes", [1, 3, 8])
@pytest.mark.parametrize("opts", [dict(), dict(fixed=True, max_iters_outer=5),
                                  dict(stop="residual", precision="mixed", outer="fcg", inner_cycles=2)])
def test_batched_equals_single_2d(lanes, opts):
    m, nb = 64, 7
    g = grid_1D(m)
    probs = [W.random_2d(m, seed=100 + b) for b in range(nb)]
    phi, cnt = solve_2d_batched(g, g, _stack(probs, "phi0"), _stack(probs, "rhs"), _stack(probs, "lam"),
                                _stack(probs, "D_xx"), _stack(probs, "D_yy"), lanes=lanes, **opts)
    assert phi.shape == (nb, m + 3, m + 3) and cnt.shape == (nb,)
    for b, p in enumerate(probs):
        one, c1 = solve_2d(g, g, *[torch.from_numpy(p[k]).to(DEV) for k in ("phi0", "rhs", "lam", "D_xx", "D_yy")],
                           **opts)
        assert torch.equal(phi[b], one), b
        assert int(cnt[b]) == int(c1), b


def test_batched_shared_and_scalar_coefficients():
    m, nb = 32, 5
    g = grid_1D(m)
    probs = [W.random_2d(m, seed=7 + b) for b in range(nb)]
    shared_D = torch.from_numpy(probs[0]["D_xx"]).to(DEV)
    phi, cnt = solve_2d_batched(g, g, _stack(probs, "phi0"), _stack(probs, "rhs"), 2.5, shared_D,
                                _stack(probs, "D_yy"), lanes=2)
    for b, p in enumerate(probs):
        one, c1 = solve_2d(g, g, torch.from_numpy(p["phi0"]).to(DEV), torch.from_numpy(p["rhs"]).to(DEV), 2.5,
                           shared_D, torch.from_numpy(p["D_yy"]).to(DEV))
        assert torch.equal(phi[b], one) and int(cnt[b]) == int(c1)
    # all-scalar D with a batched lambda
    phi, cnt = solve_2d_batched(g, g, _stack(probs, "phi0"), _stack(probs, "rhs"), _stack(probs, "lam"), 1.0, 1.0)
    for b, p in enumerate(probs):
        one, c1 = solve_2d(g, g, torch.from_numpy(p["phi0"]).to(DEV), torch.from_numpy(p["rhs"]).to(DEV),
                           torch.from_numpy(p["lam"]).to(DEV), 1.0, 1.0)
        assert torch.equal(phi[b], one) and int(cnt[b]) == int(c1)


def test_batched_matches_oracle_2d():
    """Dynamic mode: each problem's phi within 1e-12 relative L2 of the C oracle's, same count."""
    from oracle import c_oracle
    m, nb = 32, 3
    g = grid_1D(m)
    probs = [W.random_2d(m, seed=40 + b) for b in range(nb)]
    keys = ("phi0", "rhs", "lam", "D_xx", "D_yy")
    phi, cnt = solve_2d_batched(g, g, *[np.stack([p[k] for p in probs]) for k in keys], lanes=2)
    assert isinstance(phi, np.ndarray) and isinstance(cnt, np.ndarray)
    for b, p in enumerate(probs):
        ref, rc, _ = c_oracle.solve((g, g), p["phi0"], p["rhs"], p["lam"], [p["D_xx"], p["D_yy"]])
        assert int(cnt[b]) == rc
        assert np.linalg.norm(phi[b] - ref) <= 1e-12 * np.linalg.norm(ref)


def test_batched_3d_equals_single():
    m, nb = 16, 4
    g = grid_1D(m)
    rng = np.random.default_rng(3)
    shp = (nb, m + 3, m + 3, m + 3)
    phi0 = np.zeros(shp)
    rhs = rng.standard_normal(shp)
    rhs[:, :2] = rhs[:, -1:] = 0
    D = np.exp(rng.standard_normal(shp) * 0.5)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)  # noqa: E731
    phi, cnt = solve_3d_batched(g, g, g, T(phi0), T(rhs), 0.5, T(D), T(D), T(D), lanes=3, fcycle=True)
    for b in range(nb):
        one, c1 = solve_3d(g, g, g, T(phi0[b]), T(rhs[b]), 0.5, T(D[b]), T(D[b]), T(D[b]), fcycle=True)
        assert torch.equal(phi[b], one) and int(cnt[b]) == int(c1)


def test_batched_workspace_lanes_and_errors():
    from jsolver_gb300 import _engine, _lib
    lib = _lib.load()
    g = grid_1D(16)
    plan = _engine.CACHE.plan(_engine.make_grid((g, g)), _engine.make_config())
    one = lib.jmg_batched_workspace_bytes(plan.handle, 1)
    assert one >= plan.workspace_bytes
    assert lib.jmg_batched_workspace_bytes(plan.handle, 4) == 4 * one
    assert lib.jmg_batched_workspace_bytes(plan.handle, 100) == 32 * one
    with pytest.raises(ValueError, match="Shape mismatch"):
        solve_2d_batched(g, g, torch.zeros(2, 19, 19, dtype=torch.float64, device=DEV),
                         torch.zeros(2, 19, 19, dtype=torch.float64, device=DEV),
                         torch.zeros(3, 19, 19, dtype=torch.float64, device=DEV), 1.0, 1.0)


def test_batched_dxy_and_w_cycles():
    """The 9-point stencil (D_xy batched per problem) and W-cycles through the batched call."""
    m, nb = 32, 3
    g = grid_1D(m)
    rng = np.random.default_rng(5)
    probs = [W.random_2d(m, seed=60 + b) for b in range(nb)]
    dxy = np.stack([0.3 * np.minimum(p["D_xx"], p["D_yy"]) * rng.uniform(-1, 1, p["D_xx"].shape) for p in probs])
    X = [_stack(probs, k) for k in ("phi0", "rhs", "lam", "D_xx", "D_yy")]
    Dxy = torch.from_numpy(dxy).to(DEV)
    for opts in (dict(fixed=True, max_iters_outer=6), dict(gamma=2, stop="residual", precision="mixed", outer="fcg")):
        phi, cnt = solve_2d_batched(g, g, *X, D_xy=Dxy, lanes=2, **opts)
        for b in range(nb):
            one, c1 = solve_2d(g, g, *[x[b] for x in X], D_xy=Dxy[b], **opts)
            assert torch.equal(phi[b], one) and int(cnt[b]) == int(c1), (opts, b)
