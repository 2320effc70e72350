"""The CPU restatement of the learned-guess network (oracle/unet.py), checked on its own.

With BF16 rounding switched off, its hand-written backward schedule (the one the GPU
follows, csrc/mg_net.cu) must give the gradients of torch autograd through the same
forward pass. The input packing and output mapping are checked on small cases by hand.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import unet as U  # noqa: E402


def test_param_layout():
    assert U.num_params() == 175536
    sl = U.layer_slices()
    assert sl[0][0] == (0, 16 * 9 * 16) and sl[-1][1][1] == U.num_params()


def test_backward_schedule_equals_autograd(monkeypatch):
    monkeypatch.setattr(U, "bf", lambda x: x)
    rng = np.random.default_rng(0)
    p = U.init_params(1)
    for _, (bs, be) in U.layer_slices():
        p[bs:be] = rng.standard_normal(be - bs) * 0.1
    res, B = 64, 2
    x = torch.zeros((B, res, res, 16), dtype=torch.float64)
    x[..., :4] = torch.from_numpy(rng.standard_normal((B, res, res, 4)))
    t = torch.from_numpy(rng.standard_normal((B, res, res)))
    loss, g, _ = U.loss_and_grads(torch.from_numpy(p.astype(np.float64)), x, t)
    pt = torch.from_numpy(p.astype(np.float64)).requires_grad_(True)
    y, _ = U.forward(pt, x)
    ref = ((y[..., 0] - t) ** 2).mean()
    ref.backward()
    assert abs(loss - float(ref)) <= 1e-12 * abs(float(ref))
    ga = pt.grad.numpy()
    assert np.linalg.norm(g - ga) <= 1e-6 * np.linalg.norm(ga)


def test_inputs_pooling_by_hand():
    m, res = 8, 4
    n = m + 3
    rhs = np.arange(n * n, dtype=np.float64).reshape(n, n)
    x, rms = U.inputs_2d(m, res, 5.0, 1.0, np.e, rhs)
    # pixel (0, 0) averages rows 1..2, columns 1..2 of the padded grid
    blk = rhs[1:3, 1:3].mean()
    pooled = rhs[1:9, 1:9].reshape(4, 2, 4, 2).mean(axis=(1, 3))
    assert rms == pytest.approx(np.sqrt(np.mean(pooled.astype(np.float32).astype(np.float64) ** 2)), rel=1e-6)
    assert x[0, 0, 0] == 0.0 and x[0, 0, 1] == 1.0 and x[0, 0, 2] == pytest.approx(0.5, rel=4e-3)
    assert x[0, 0, 3] == pytest.approx(blk / rms, rel=8e-3)
    assert np.all(x[..., 4:] == 0)


def test_output_mapping_identity_at_full_resolution():
    m = res = 8
    y = np.arange(res * res, dtype=np.float64).reshape(res, res)
    phi = U.output_2d(y, 2.0, 0.5, m)
    # f = 1: phi[1 + a, 1 + b] = y[a, b] on the interior, frame zero
    assert np.allclose(phi[2:m + 1, 2:m + 1], y[1:m, 1:m])
    assert np.all(phi[:2] == 0) and np.all(phi[m + 1:] == 0) and np.all(phi[:, :2] == 0)
