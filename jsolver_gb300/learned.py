"""Learned initial guess for 2D solves: a small U-Net run and trained by this library's kernels.

The reference always starts from the caller's phi0 (zero in its benchmarks). Here a
4-level U-Net (16/32/64/64 channels, 3x3 convolutions, BF16 weights and activations,
FP32 accumulation on the tensor cores; csrc/mg_net.cu) predicts phi0 from
(log D_xx, log D_yy, lambda, rhs) on a 256^2 network grid; finer grids are averaged
onto it and the prediction is interpolated back bilinearly. The multigrid then
iterates from the guess to the caller's tolerance, so its residual judges the guess
and a poor guess only costs cycles.

Training data: random problems with the coefficients of the 2D random-coefficient
workload (D_xx, D_yy = exp(GRF sigma 1, correlation length 0.05), lambda ~ U[0, 10])
and rhs = L_h phi* for a random smooth phi* (a random combination of low sine modes,
of which the workload's sin(pi x) sin(2 pi y) is one member); the targets are the
plain FP64 multigrid's solutions of those problems. Problems are sampled on the GPU
with torch (plumbing only: random fields and the manufactured rhs); every solve,
forward pass, gradient and optimiser step runs in libjmg.

Command line (on a GPU machine):  python -m jsolver_gb300.learned train --out PATH
"""
import argparse
import ctypes
import json
import math
import os
import time

import numpy as np
import torch

from . import _engine, _lib
from .grid_1d import grid_1D

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights", "unet_guess_256.npz")


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def num_params():
    return int(_lib.load().jmg_net_num_params())


class GuessNet:
    """The network on one GPU (a JmgNet handle plus its parameters)."""

    def __init__(self, res=256, max_batch=1, device=None, params=None, out_scale=1.0):
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.res = int(res)
        self.max_batch = int(max_batch)
        self.out_scale = float(out_scale)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_create(ctypes.byref(h), self.res, self.max_batch))
        self.handle = h
        self.rms = torch.zeros(1, dtype=torch.float32, device=self.device)
        if params is not None:
            self.set_params(params)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.lib.jmg_net_destroy(h)
            self.handle = None

    # parameters ---------------------------------------------------------------------
    def set_params(self, params):
        p = torch.as_tensor(np.asarray(params, dtype=np.float32) if not isinstance(params, torch.Tensor) else params,
                            dtype=torch.float32).to(self.device).contiguous()
        if p.numel() != num_params():
            raise ValueError(f"expected {num_params()} parameters, got {p.numel()}")
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_set_params(self.handle, _p(p), _stream(self.device)))
            torch.cuda.current_stream(self.device).synchronize()

    def get_params(self):
        p = torch.empty(num_params(), dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_get_params(self.handle, _p(p), _stream(self.device)))
        return p

    @classmethod
    def load(cls, path=WEIGHTS, max_batch=1, device=None):
        z = np.load(path)
        return cls(res=int(z["res"]), max_batch=max_batch, device=device, params=z["params"],
                   out_scale=float(z["out_scale"]))

    def save(self, path, **meta):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez(path, params=self.get_params().cpu().numpy(), out_scale=np.float64(self.out_scale),
                 res=np.int64(self.res), meta=json.dumps(meta))

    # network calls --------------------------------------------------------------------
    def forward(self, x):
        """x: bf16 [B, res, res, 16] on the device -> y float32 [B, res, res]."""
        B = x.shape[0]
        y = torch.empty((B, self.res, self.res), dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_forward(self.handle, _p(x), B, _p(y), _stream(self.device)))
        return y

    def loss_grad(self, x, target):
        B = x.shape[0]
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        g = torch.empty(num_params(), dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_loss_grad(self.handle, _p(x), _p(target), B, _p(loss), _p(g),
                                                  _stream(self.device)))
        return loss, g

    def train_step(self, x, target, lr, loss=None):
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_train_step(self.handle, _p(x), _p(target), x.shape[0], ctypes.c_float(lr),
                                                   _p(loss), _stream(self.device)))

    # solver-side inputs and outputs ---------------------------------------------------
    def _coeffs(self, gx, gy, rhs, lam, D_xx, D_yy):
        grid = _engine.make_grid((gx, gy))
        sl, spatial, _ = _engine.validate(2, rhs, rhs, lam, (D_xx, D_yy), None, _engine.expected_shape((gx, gy)))
        prep = _engine.Prepared(2, self.device, lam, (D_xx, D_yy), None, sl, spatial)
        return grid, prep

    def inputs(self, gx, gy, rhs, lam, D_xx, D_yy, x_out=None):
        """Packed input of one problem (bf16 [res, res, 16]) and its rhs RMS (device)."""
        grid, prep = self._coeffs(gx, gy, rhs, lam, D_xx, D_yy)
        r = _engine.to_device(rhs, self.device)
        x = x_out if x_out is not None else torch.empty((self.res, self.res, 16), dtype=torch.bfloat16,
                                                         device=self.device)
        rms = torch.empty(1, dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_inputs_2d(self.handle, ctypes.byref(grid), ctypes.byref(prep.coeffs), _p(r),
                                                  _p(x), _p(rms), _stream(self.device)))
        return x, rms

    def target(self, gx, gy, phi, rms, out=None):
        grid = _engine.make_grid((gx, gy))
        ph = _engine.to_device(phi, self.device)
        t = out if out is not None else torch.empty((self.res, self.res), dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_target_2d(self.handle, ctypes.byref(grid), _p(ph), _p(rms),
                                                  ctypes.c_float(self.out_scale), _p(t), _stream(self.device)))
        return t

    def guess(self, gx, gy, rhs, lam, D_xx, D_yy):
        """phi0 (float64, padded (m+3)^2, zero frame) for one problem."""
        grid, prep = self._coeffs(gx, gy, rhs, lam, D_xx, D_yy)
        r = _engine.to_device(rhs, self.device)
        phi0 = torch.empty_like(r)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jmg_net_guess_2d(self.handle, ctypes.byref(grid), ctypes.byref(prep.coeffs), _p(r),
                                                 ctypes.c_float(self.out_scale), _p(phi0), _stream(self.device)))
        return phi0


_DEFAULT = {}


def default_net(device):
    """The package's trained network on `device` (loaded once per device)."""
    key = str(device)
    if key not in _DEFAULT:
        if not os.path.exists(WEIGHTS):
            raise FileNotFoundError(f"no trained weights at {WEIGHTS}: train them with "
                                    "`python -m jsolver_gb300.learned train`")
        _DEFAULT[key] = GuessNet.load(WEIGHTS, device=device)
    return _DEFAULT[key]


def predict_phi0(guess, grids, rhs, lam, D, device):
    """phi0 from the network ('learned' = the package's weights, or a GuessNet)."""
    net = default_net(device) if isinstance(guess, str) and guess == "learned" else guess
    if not isinstance(net, GuessNet):
        raise ValueError("guess must be None, 'learned' or a GuessNet")
    gx, gy = grids
    return net.guess(gx, gy, rhs, lam, D[0], D[1])


# ---- problem sampling (torch on the GPU; the distributions of workloads.random_2d) ------

def _grf(n, shape, h, corr_len, sigma, gen, device):
    """Batch of zero-mean, unit-std Gaussian random fields (Gaussian covariance), periodic."""
    white = torch.randn((n,) + shape, generator=gen, device=device, dtype=torch.float64)
    f = torch.fft.rfft2(white)
    ky = torch.fft.fftfreq(shape[0], d=h, device=device, dtype=torch.float64) * 2 * math.pi
    kx = torch.fft.rfftfreq(shape[1], d=h, device=device, dtype=torch.float64) * 2 * math.pi
    k2 = ky[:, None] ** 2 + kx[None, :] ** 2
    g = torch.fft.irfft2(f * torch.exp(-0.25 * k2 * corr_len ** 2), s=shape)
    g = g - g.mean(dim=(1, 2), keepdim=True)
    g = g / g.std(dim=(1, 2), keepdim=True, unbiased=False)
    return sigma * g


def apply_operator_2d(phi, Dxx, Dyy, lam, idel):
    """Batched L_h phi on interior indices 2..m (workloads.apply_operator_2d)."""
    Dx, Dy = Dxx.clone(), Dyy.clone()
    Dx[:, 1:-1, :-1] = 0.5 * (Dxx[:, 1:-1, 1:] + Dxx[:, 1:-1, :-1])
    Dy[:, :-1, 1:-1] = 0.5 * (Dyy[:, 1:, 1:-1] + Dyy[:, :-1, 1:-1])
    s = idel ** 2
    out = torch.zeros_like(phi)
    i = slice(2, -2)
    lc, rc = Dx[:, i, 1:-3] * s, Dx[:, i, 2:-2] * s
    cl, cr = Dy[:, 1:-3, i] * s, Dy[:, 2:-2, i] * s
    cc = lc + rc + cl + cr + lam[:, i, i]
    out[:, i, i] = (lc * phi[:, i, 1:-3] + rc * phi[:, i, 3:-1] + cl * phi[:, 1:-3, i] + cr * phi[:, 3:-1, i]
                    - cc * phi[:, i, i])
    return out


def sample_problems(n, m, seed, device, phi_kind="modes", modes=6):
    """n problems on an m x m grid. phi_kind 'modes': random smooth phi* (training);
    'workload': phi* = sin(pi x) sin(2 pi y) as in the 2D random-coefficient workload."""
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    N = m + 3
    h = 1.0 / m
    Dxx = torch.exp(_grf(n, (N, N), h, 0.05, 1.0, gen, device))
    Dyy = torch.exp(_grf(n, (N, N), h, 0.05, 1.0, gen, device))
    lam = 10.0 * torch.rand((n, N, N), generator=gen, device=device, dtype=torch.float64)
    c = (torch.arange(N, device=device, dtype=torch.float64) - 1.0) * h  # grid_1D(m).centers
    if phi_kind == "workload":
        phi = (torch.sin(math.pi * c)[None, :] * torch.sin(2 * math.pi * c)[:, None]).expand(n, N, N).clone()
    else:
        k = torch.arange(1, modes + 1, device=device, dtype=torch.float64)
        sx = torch.sin(math.pi * k[:, None] * c[None, :])  # [modes, N] along x
        amp = torch.randn((n, modes, modes), generator=gen, device=device, dtype=torch.float64)
        amp = amp / (k[:, None] ** 2 + k[None, :] ** 2)
        phi = torch.einsum("bkl,ky,lx->byx", amp, sx, sx)
    phi[:, :2, :] = 0
    phi[:, -2:, :] = 0
    phi[:, :, :2] = 0
    phi[:, :, -2:] = 0
    rhs = apply_operator_2d(phi, Dxx, Dyy, lam, float(m))
    return dict(D_xx=Dxx, D_yy=Dyy, lam=lam, rhs=rhs, phi_exact=phi)


# ---- dataset, training, evaluation --------------------------------------------------------

def solve_plain(g, prob, i, rtol=1e-10, precision="fp64", phi0=None, outer="richardson"):
    from .solver_2d import solve_2d
    rhs = prob["rhs"][i]
    p0 = torch.zeros_like(rhs) if phi0 is None else phi0
    return solve_2d(g, g, p0, rhs, prob["lam"][i], prob["D_xx"][i], prob["D_yy"][i], stop="residual", rtol=rtol,
                    precision=precision, outer=outer)


def build_dataset(net, n, m=256, seed=1, chunk=250, rtol=1e-8, log=print):
    """Inputs X (bf16 [n, res, res, 16]) and targets T (float32 [n, res, res]) from plain
    FP64 multigrid solutions of sampled problems; sets net.out_scale from the first chunk."""
    g = grid_1D(m)
    dev = net.device
    X = torch.empty((n, net.res, net.res, 16), dtype=torch.bfloat16, device=dev)
    T = torch.empty((n, net.res, net.res), dtype=torch.float32, device=dev)
    t0 = time.time()
    cycles = []
    for c0 in range(0, n, chunk):
        k = min(chunk, n - c0)
        prob = sample_problems(k, m, seed * 1000003 + c0, dev)
        sols, rmss = [], []
        for i in range(k):
            phi, cnt = solve_plain(g, prob, i, rtol=rtol)
            cycles.append(int(cnt))
            _, rms = net.inputs(g, g, prob["rhs"][i], prob["lam"][i], prob["D_xx"][i], prob["D_yy"][i], x_out=X[c0 + i])
            sols.append(phi)
            rmss.append(rms)
        if c0 == 0:
            # output scale: median ratio of the solution's RMS to the pooled rhs RMS
            f = m // net.res
            ratios = []
            for phi, rms in zip(sols, rmss):
                pb = phi[1:1 + f * net.res, 1:1 + f * net.res].reshape(net.res, f, net.res, f).mean(dim=(1, 3))
                ratios.append(float(pb.pow(2).mean().sqrt()) / float(rms))
            net.out_scale = float(np.median(ratios))
        for i in range(k):
            net.target(g, g, sols[i], rmss[i], out=T[c0 + i])
        if log and (c0 // chunk) % 8 == 0:
            log(f"dataset {c0 + k}/{n}  {time.time() - t0:.1f}s  median cycles {int(np.median(cycles))}")
    torch.cuda.synchronize(dev)
    return X, T, dict(seconds=time.time() - t0, median_cycles=float(np.median(cycles)), out_scale=net.out_scale)


def train(net, X, T, epochs=10, batch=32, lr=2e-3, lr_min=2e-5, seed=0, val=None, log=print):
    """Adam with cosine learning-rate decay over shuffled mini-batches."""
    n = X.shape[0]
    steps = epochs * (n // batch)
    gen = torch.Generator(device=net.device)
    gen.manual_seed(seed)
    loss = torch.zeros(1, dtype=torch.float32, device=net.device)
    hist = []
    t0 = time.time()
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen, device=net.device)
        loss.zero_()
        nb = n // batch
        for b in range(nb):
            idx = perm[b * batch:(b + 1) * batch]
            xb, tb = X.index_select(0, idx), T.index_select(0, idx)
            a = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * step / max(steps, 1)))
            net.train_step(xb, tb, a, loss)
            step += 1
        ep_loss = float(loss.item()) / nb
        rec = dict(epoch=ep, train_mse=ep_loss, seconds=time.time() - t0)
        if val is not None:
            rec["val_mse"] = val_mse(net, *val)
        hist.append(rec)
        if log:
            log(json.dumps(rec))
    return hist


def val_mse(net, X, T, batch=32):
    tot, cnt = 0.0, 0
    for b in range(0, X.shape[0], batch):
        xb, tb = X[b:b + batch], T[b:b + batch]
        y = net.forward(xb)
        tot += float(((y - tb) ** 2).sum())
        cnt += tb.numel()
    return tot / cnt


def evaluate(net, m, seeds, phi_kind="workload", rtol=1e-10,
             forms=(("fp64", "richardson"), ("mixed", "richardson"), ("mixed", "fcg"))):
    """Cycles, solve times and initial residuals from the zero guess and from the
    learned guess on held-out problems (one problem per seed)."""
    g = grid_1D(m)
    dev = net.device
    rows = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for s in seeds:
        prob = sample_problems(1, m, s, dev, phi_kind=phi_kind)
        rhs, lam, dxx, dyy = prob["rhs"][0], prob["lam"][0], prob["D_xx"][0], prob["D_yy"][0]
        row = dict(seed=int(s))
        ev0.record()
        phi0 = net.guess(g, g, rhs, lam, dxx, dyy)
        ev1.record()
        ev1.synchronize()
        row["guess_ms"] = ev0.elapsed_time(ev1)
        row["guess_rel_residual"] = rel_residual(g, phi0, rhs, lam, dxx, dyy)
        row["guess_rel_err"] = float((phi0 - prob["phi_exact"][0]).norm() / prob["phi_exact"][0].norm())
        for prec, outer in forms:
            for name, start in (("zero", None), ("learned", phi0)):
                ev0.record()
                if start is None:
                    phi, cnt = solve_plain(g, prob, 0, rtol=rtol, precision=prec, outer=outer)
                else:
                    phi0b = net.guess(g, g, rhs, lam, dxx, dyy)
                    phi, cnt = solve_plain(g, prob, 0, rtol=rtol, precision=prec, phi0=phi0b, outer=outer)
                ev1.record()
                ev1.synchronize()
                row[f"{prec}-{outer}_{name}_cycles"] = int(cnt)
                row[f"{prec}-{outer}_{name}_ms"] = ev0.elapsed_time(ev1)
        rows.append(row)
    return rows


def rel_residual(g, phi, rhs, lam, dxx, dyy):
    """||rhs - L_h phi|| / ||rhs|| (FP64, on the GPU) of one 2D problem."""
    from ._engine import OperatorSet
    ops = OperatorSet((g, g), lam, (dxx, dyy))
    return float(ops.rel_residual(phi, rhs))


def summarise(rows):
    keys = [k for k in rows[0] if k != "seed"]
    out = {}
    for k in keys:
        v = np.array([r[k] for r in rows], dtype=np.float64)
        out[k] = dict(median=float(np.median(v)), p10=float(np.percentile(v, 10)), p90=float(np.percentile(v, 90)),
                      mean=float(v.mean()))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", default=WEIGHTS)
    t.add_argument("--n", type=int, default=20000)
    t.add_argument("--n-val", type=int, default=512)
    t.add_argument("--epochs", type=int, default=10)
    t.add_argument("--batch", type=int, default=32)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--seed", type=int, default=1)
    t.add_argument("--log", default=None)
    e = sub.add_parser("eval")
    e.add_argument("--weights", default=WEIGHTS)
    e.add_argument("--m", type=int, default=256)
    e.add_argument("--seeds", type=int, default=1000)
    e.add_argument("--first-seed", type=int, default=10 ** 8)
    e.add_argument("--phi", default="workload", choices=["workload", "modes"])
    e.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    logf = open(a.log, "a") if getattr(a, "log", None) else None

    def log(msg):
        print(msg, flush=True)
        if logf:
            logf.write(msg + "\n")
            logf.flush()

    if a.cmd == "train":
        net = GuessNet(res=256, max_batch=a.batch, device=dev)
        net.set_params(init_params(a.seed))
        X, T, info = build_dataset(net, a.n + a.n_val, seed=a.seed, log=log)
        log(json.dumps(dict(dataset=info)))
        n = a.n
        hist = train(net, X[:n], T[:n], epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed,
                     val=(X[n:], T[n:]), log=log)
        net.save(a.out, dataset=info, history=hist, n_train=n, n_val=a.n_val, epochs=a.epochs, batch=a.batch,
                 lr=a.lr, seed=a.seed)
        log(f"saved {a.out}")
    else:
        net = GuessNet.load(a.weights, device=dev)
        seeds = range(a.first_seed, a.first_seed + a.seeds)
        rows = evaluate(net, a.m, seeds, phi_kind=a.phi)
        res = dict(m=a.m, phi=a.phi, n=len(rows), summary=summarise(rows))
        log(json.dumps(res))
        if a.out:
            with open(a.out, "w") as f:
                json.dump(dict(res, rows=rows), f)
    return 0


def init_params(seed=0):
    """He-normal weights (fan-in 9 cin) for the ReLU layers, zero biases; the linear
    output layer starts 10x smaller so the first guesses are near zero."""
    layers = [(16, 16, 1), (16, 16, 1), (16, 32, 1), (32, 32, 1), (32, 64, 1), (64, 64, 1), (64, 64, 1), (64, 64, 1),
              (64, 32, 1), (32, 16, 1), (16, 16, 1), (16, 16, 0)]
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co, relu in layers:
        std = math.sqrt(2.0 / (9 * ci)) * (1.0 if relu else 0.1)
        parts.append(rng.standard_normal(co * 9 * ci) * std)
        parts.append(np.zeros(co))
    return np.concatenate(parts).astype(np.float32)


if __name__ == "__main__":
    raise SystemExit(main())
