"""torch.library operators over the C ABI (jsolver_gb300.torch_ops): registration and
fake (shape-only) kernels on the CPU; on the GPU the operators give solve_2d's and
solve_3d's bits and pass torch.library.opcheck."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from jsolver_gb300 import torch_ops  # noqa: E402,F401  (registers the operators)
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402


def test_operators_registered():
    assert hasattr(torch.ops.jmg, "solve_2d") and hasattr(torch.ops.jmg, "solve_3d")
    s = str(torch.ops.jmg.solve_2d.default._schema)
    assert "Tensor? D_xy" in s and "str precision" in s


def test_fake_kernels_give_shapes():
    from torch._subclasses.fake_tensor import FakeTensorMode
    g = grid_1D(16)
    with FakeTensorMode():
        a = torch.empty(19, 19, dtype=torch.float64)
        phi, c = torch.ops.jmg.solve_2d(a, a, a, a, a, None, *torch_ops.grid_args(g, g), *torch_ops.options())
        assert phi.shape == (19, 19) and phi.dtype == torch.float64 and c.shape == () and c.dtype == torch.int64
        b = torch.empty(11, 11, 11, dtype=torch.float64)
        g3 = grid_1D(8)
        phi, c = torch.ops.jmg.solve_3d(b, b, b, b, b, b, *torch_ops.grid_args(g3, g3, g3),
                                        *torch_ops.options(fcycle=True))
        assert phi.shape == (11, 11, 11) and c.dtype == torch.int64


def test_options_order_matches_solve_2d_keywords():
    import inspect
    from jsolver_gb300.solver_2d import solve_2d
    params = inspect.signature(solve_2d).parameters
    for name, value in zip(torch_ops._OPTION_NAMES, torch_ops.options()):
        assert params[name].default == value, name


@pytest.mark.gpu
def test_operators_match_solve_and_opcheck():
    if not torch.cuda.is_available():  # pragma: no cover
        pytest.skip("needs a CUDA GPU")
    from jsolver_gb300 import workloads as W
    from jsolver_gb300.solver_2d import solve_2d
    from jsolver_gb300.solver_3d import solve_3d
    dev = torch.device("cuda", 0)
    g = grid_1D(64)
    p = W.random_2d(64, seed=3)
    args = [torch.from_numpy(p[k]).to(dev) for k in ("phi0", "rhs", "lam", "D_xx", "D_yy")]
    for opts in (dict(), dict(stop="residual", precision="mixed", outer="fcg", inner_cycles=2),
                 dict(fixed=True, max_iters_outer=4)):
        phi, c = torch.ops.jmg.solve_2d(*args, None, *torch_ops.grid_args(g, g), *torch_ops.options(**opts))
        ref, rc = solve_2d(g, g, *args, **opts)
        assert torch.equal(phi, ref) and int(c) == int(rc)
    lam0 = torch.tensor(0.5, dtype=torch.float64, device=dev)  # a 0-d tensor is a scalar
    phi, c = torch.ops.jmg.solve_2d(args[0], args[1], lam0, args[3], args[4], None, *torch_ops.grid_args(g, g),
                                    *torch_ops.options())
    ref, rc = solve_2d(g, g, args[0], args[1], 0.5, args[3], args[4])
    assert torch.equal(phi, ref) and int(c) == int(rc)
    # host tensors: solved on the GPU, returned on the host
    cpu = [a.cpu() for a in args]
    phi, c = torch.ops.jmg.solve_2d(*cpu, None, *torch_ops.grid_args(g, g), *torch_ops.options())
    ref, rc = solve_2d(g, g, *args)
    assert phi.device.type == "cpu" and c.device.type == "cpu"
    assert torch.equal(phi, ref.cpu()) and int(c) == int(rc)
    torch.library.opcheck(torch.ops.jmg.solve_2d.default,
                          (*args, None, *torch_ops.grid_args(g, g), *torch_ops.options()),
                          test_utils=("test_schema", "test_faketensor"))
    g3 = grid_1D(16)
    rng = np.random.default_rng(1)
    b = [torch.from_numpy(x).to(dev) for x in (np.zeros((19,) * 3), rng.standard_normal((19,) * 3), np.ones((19,) * 3))]
    phi, c = torch.ops.jmg.solve_3d(b[0], b[1], b[2], b[2], b[2], b[2], *torch_ops.grid_args(g3, g3, g3),
                                    *torch_ops.options(fcycle=True))
    ref, rc = solve_3d(g3, g3, g3, b[0], b[1], b[2], b[2], b[2], b[2], fcycle=True)
    assert torch.equal(phi, ref) and int(c) == int(rc)
