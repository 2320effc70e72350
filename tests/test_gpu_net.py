"""Learned initial guess: the GPU network (libjmg) against its CPU restatement (oracle/unet.py).

The oracle rounds to BF16 at the same points as the GPU (stored activations and
activation gradients); the GPU differs in the order of its FP32 sums (tensor-core tiles,
atomics), which flips an occasional BF16 rounding. Tolerances: forward output 1e-2
relative L2, loss 1e-3 relative, each layer's weight and bias gradients 3e-2 relative L2.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from jsolver_gb300 import learned as LN  # noqa: E402
from jsolver_gb300.grid_1d import grid_1D  # noqa: E402
from jsolver_gb300.solver_2d import solve_2d  # noqa: E402
from oracle import unet as U  # noqa: E402

DEV = torch.device("cuda", 0)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def _params(seed):
    p = U.init_params(seed)
    rng = np.random.default_rng(seed + 1)
    for (ws, we), (bs, be) in U.layer_slices():
        p[bs:be] = rng.standard_normal(be - bs).astype(np.float32) * 0.05
    # a larger output layer so that the loss gradient is not dominated by rounding
    (ws, we), _ = U.layer_slices()[-1]
    p[ws:we] *= 10
    return p


def _inputs(B, res, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((B, res, res, 16), np.float32)
    x[..., :4] = rng.standard_normal((B, res, res, 4)).astype(np.float32)
    xb = U.bf(torch.from_numpy(x))
    return xb, xb.to(torch.bfloat16).to(DEV)


def test_param_count():
    assert LN.num_params() == U.num_params()


def test_forward_matches_oracle():
    res, B = 128, 2
    p = _params(0)
    net = LN.GuessNet(res=res, max_batch=B, device=DEV, params=p)
    xo, xg = _inputs(B, res, 1)
    y = net.forward(xg).cpu().numpy()
    yo, _ = U.forward(p, xo)
    r = rel(y, yo[..., 0].numpy())
    assert r < 1e-2, r


def test_gradients_match_oracle():
    res, B = 128, 2
    p = _params(2)
    net = LN.GuessNet(res=res, max_batch=B, device=DEV, params=p)
    xo, xg = _inputs(B, res, 3)
    rng = np.random.default_rng(4)
    t = rng.standard_normal((B, res, res)).astype(np.float32)
    loss, g = net.loss_grad(xg, torch.from_numpy(t).to(DEV))
    lo, go, _ = U.loss_and_grads(p, xo, torch.from_numpy(t))
    assert abs(float(loss) - lo) <= 1e-3 * abs(lo)
    g = g.cpu().numpy()
    for li, ((ws, we), (bs, be)) in enumerate(U.layer_slices()):
        assert rel(g[ws:we], go[ws:we]) < 3e-2, (li, "W", rel(g[ws:we], go[ws:we]))
        if np.linalg.norm(go[bs:be]) > 0:
            assert rel(g[bs:be], go[bs:be]) < 3e-2, (li, "b", rel(g[bs:be], go[bs:be]))


def test_train_steps_reduce_loss():
    res, B = 128, 4
    net = LN.GuessNet(res=res, max_batch=B, device=DEV, params=LN.init_params(5))
    _, xg = _inputs(B, res, 6)
    yy, xx = np.meshgrid(np.linspace(0, 1, res), np.linspace(0, 1, res), indexing="ij")
    t = torch.from_numpy(np.broadcast_to(np.sin(np.pi * xx) * np.sin(2 * np.pi * yy), (B, res, res))
                         .astype(np.float32).copy()).to(DEV)
    l0, _ = net.loss_grad(xg, t)
    for _ in range(200):
        net.train_step(xg, t, 2e-3)
    l1, _ = net.loss_grad(xg, t)
    assert float(l1) < 0.5 * float(l0), (float(l0), float(l1))


@pytest.mark.parametrize("m,res", [(256, 256), (512, 256), (256, 128)])
def test_inputs_and_guess_mapping(m, res):
    prob = LN.sample_problems(1, m, 7, DEV)
    g = grid_1D(m)
    p = _params(8)
    net = LN.GuessNet(res=res, max_batch=1, device=DEV, params=p, out_scale=0.02)
    args = [prob[k][0] for k in ("rhs", "lam", "D_xx", "D_yy")]
    x, rms = net.inputs(g, g, *args)
    xo, rmso = U.inputs_2d(m, res, *[a.cpu().numpy() for a in (args[1], args[2], args[3], args[0])])
    assert abs(float(rms) - rmso) <= 1e-6 * rmso
    xg = x.float().cpu().numpy()
    assert np.allclose(xg, xo, rtol=8e-3, atol=1e-6), np.abs(xg - xo).max()
    phi0 = net.guess(g, g, *args).cpu().numpy()
    y = net.forward(x[None]).cpu().numpy()[0]
    ref = U.output_2d(y, rmso, 0.02, m)
    beta = U.ritz_scale(ref, *[a.cpu().numpy() for a in (args[0], args[1], args[2], args[3])], m)
    assert rel(phi0, beta * ref) < 1e-6, rel(phi0, beta * ref)


WEIGHTS = LN.WEIGHTS


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights in the package")
@pytest.mark.parametrize("m", [256, 1024])
def test_trained_guess_against_zero_guess(m):
    """The committed network against the zero guess on held-out problems of the 2D
    random-coefficient workload (seeds outside the training range). Both starts reach
    relative residual 1e-10 through the plain multigrid, which judges the guess; the
    cycle counts are measured and reported, not assumed: with this smoother and its
    injected coarse operators, guess errors of a fraction of a percent in the slow
    modes cost cycles (tests/test_guess_error_modes.py)."""
    net = LN.GuessNet.load(WEIGHTS, device=DEV)
    g = grid_1D(m)
    zero, learned, err = [], [], []
    for s in range(4):
        prob = LN.sample_problems(1, m, 10 ** 7 + s, DEV, phi_kind="workload")
        args = [prob[k][0] for k in ("rhs", "lam", "D_xx", "D_yy")]
        phi0 = net.guess(g, g, *args)
        err.append(float((phi0 - prob["phi_exact"][0]).norm() / prob["phi_exact"][0].norm()))
        phi_z, c0 = LN.solve_plain(g, prob, 0)
        phi_l, c1 = LN.solve_plain(g, prob, 0, phi0=phi0)
        for phi in (phi_z, phi_l):
            assert LN.rel_residual(g, phi, *args) <= 1e-10
        zero.append(int(c0))
        learned.append(int(c1))
    print(f"m={m}: guess rel. error {np.median(err):.3f}; cycles zero {zero} learned {learned}")
    assert np.median(err) < 1.0  # the Ritz-scaled guess is closer to phi than zero is


@pytest.mark.parametrize("res,B", [(128, 2), (256, 8)])
def test_tcgen05_convolutions_match_mma_sync(res, B, monkeypatch):
    """The convolutions on the 5th-generation tensor cores (tcgen05.mma into tensor memory,
    TMA input tiles; the default) against the mma.sync kernels (JMG_CONV=mma): the same
    network output and gradients up to the order of the FP32 sums, which flips an
    occasional BF16 rounding of a stored activation (forward 5e-3, gradients 2e-2
    relative L2)."""
    p = _params(5)
    xo, xg = _inputs(B, res, 6)
    t = torch.from_numpy(np.random.default_rng(7).standard_normal((B, res, res)).astype(np.float32)).to(DEV)
    out = {}
    for kind in ("mma", "tc"):
        if kind == "mma":
            monkeypatch.setenv("JMG_CONV", "mma")
        else:
            monkeypatch.delenv("JMG_CONV", raising=False)
        net = LN.GuessNet(res=res, max_batch=B, device=DEV, params=p)
        y = net.forward(xg).cpu().numpy()
        loss, g = net.loss_grad(xg, t)
        out[kind] = (y, float(loss), g.cpu().numpy())
    (y0, l0, g0), (y1, l1, g1) = out["mma"], out["tc"]
    assert rel(y1, y0) < 5e-3, rel(y1, y0)
    assert abs(l1 - l0) <= 1e-3 * abs(l0)
    for li, ((ws, we), (bs, be)) in enumerate(U.layer_slices()):
        assert rel(g1[ws:we], g0[ws:we]) < 2e-2, (li, rel(g1[ws:we], g0[ws:we]))
