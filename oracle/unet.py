"""CPU restatement of the learned-guess network (test infrastructure only).

Checks the GPU network of jsolver_gb300 (csrc/mg_net.cu, csrc/net_kernels.cuh): the same
U-Net, parameter layout, input packing and output mapping, with BF16 rounding at the
same points as the GPU (activations and activation gradients are stored in BF16, every
sum is formed in FP32). The GPU differs only in the order of FP32 accumulation (tensor-
core MMA tiles, atomics), so outputs agree to a few BF16 ulps and gradients to ~1e-3.
The reference has no learned part; this file is the oracle for it, not a port.

Parameters: per layer the weights [cout][3][3][cin] then the bias [cout] (FP32).
Activations: NHWC float32 tensors whose values are BF16-representable.
"""
import numpy as np
import torch
import torch.nn.functional as F

# (cin, cout, level, relu)
LAYERS = [(16, 16, 0, 1), (16, 16, 0, 1), (16, 32, 1, 1), (32, 32, 1, 1), (32, 64, 2, 1), (64, 64, 2, 1),
          (64, 64, 3, 1), (64, 64, 3, 1), (64, 32, 2, 1), (32, 16, 1, 1), (16, 16, 0, 1), (16, 16, 0, 0)]


def num_params():
    return sum(co * 9 * ci + co for ci, co, _, _ in LAYERS)


def split_params(p):
    """Flat vector -> list of (W [cout,3,3,cin], b [cout]) torch tensors (a torch tensor
    stays as it is, so autograd can follow it; anything else becomes FP32)."""
    if not isinstance(p, torch.Tensor):
        p = torch.as_tensor(np.asarray(p, dtype=np.float32))
    out, o = [], 0
    for ci, co, _, _ in LAYERS:
        w = p[o:o + co * 9 * ci].reshape(co, 3, 3, ci)
        o += co * 9 * ci
        b = p[o:o + co]
        o += co
        out.append((w, b))
    return out


def init_params(seed=0):
    """He-normal weights for ReLU layers (fan-in 9 cin), zero biases; the output layer
    is scaled down so that the initial guess starts near zero."""
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co, _, relu in LAYERS:
        std = np.sqrt(2.0 / (9 * ci)) * (1.0 if relu else 0.1)
        parts.append(rng.standard_normal(co * 9 * ci) * std)
        parts.append(np.zeros(co))
    return np.concatenate(parts).astype(np.float32)


def bf(x):
    return x.to(torch.bfloat16).to(torch.float32)


def _conv(x, w, b):
    # x [N,H,W,C]; cross-correlation with zero padding 1, tap (dh, dw) reads (y+dh-1, x+dw-1)
    y = F.conv2d(x.permute(0, 3, 1, 2), w.permute(0, 3, 1, 2), bias=b, padding=1)
    return y.permute(0, 2, 3, 1)


def _pool(x):
    return bf(0.25 * (((x[:, 0::2, 0::2] + x[:, 0::2, 1::2]) + x[:, 1::2, 0::2]) + x[:, 1::2, 1::2]))


def _up(x):
    return x.repeat_interleave(2, dim=1).repeat_interleave(2, dim=2)


def forward(params, x):
    """x: [N,H,W,16] (BF16 values). Returns (y [N,H,W,16] FP32, dict of activations)."""
    P = split_params(params)
    P = [(bf(w), b) for w, b in P]
    a = {}

    def L(i, inp):
        w, b = P[i]
        y = _conv(inp, w, b)
        if LAYERS[i][3]:
            return bf(torch.clamp_min(y, 0.0))
        return y

    a["x"] = x
    a[0] = L(0, x)
    a[1] = L(1, a[0])
    a["p0"] = _pool(a[1])
    a[2] = L(2, a["p0"])
    a[3] = L(3, a[2])
    a["p1"] = _pool(a[3])
    a[4] = L(4, a["p1"])
    a[5] = L(5, a[4])
    a["p2"] = _pool(a[5])
    a[6] = L(6, a["p2"])
    a[7] = L(7, a[6])
    a["u2"] = bf(_up(a[7]) + a[5])
    a[8] = L(8, a["u2"])
    a["u1"] = bf(_up(a[8]) + a[3])
    a[9] = L(9, a["u1"])
    a["u0"] = bf(_up(a[9]) + a[1])
    a[10] = L(10, a["u0"])
    y = L(11, a[10])
    return y, a


def loss_and_grads(params, x, target):
    """Mean squared error of channel 0 against target [N,H,W] and its gradient with
    respect to the flat parameter vector, following the GPU's backward schedule."""
    P = split_params(params)
    Pb = [(bf(w), b) for w, b in P]
    y, a = forward(params, x)
    npix = target.numel()
    d = y[..., 0] - target
    loss = float((d * d).sum() / npix)
    gy = torch.zeros_like(y)
    gy[..., 0] = bf(2.0 * d / npix)
    grads = [None] * len(LAYERS)

    def back(i, inp, gout, mask):
        w, _ = Pb[i]
        gw = torch.nn.grad.conv2d_weight(inp.permute(0, 3, 1, 2), w.permute(0, 3, 1, 2).shape,
                                         gout.permute(0, 3, 1, 2), padding=1)
        grads[i] = (gw.permute(0, 2, 3, 1).contiguous(), gout.sum(dim=(0, 1, 2)))
        gin = torch.nn.grad.conv2d_input(inp.permute(0, 3, 1, 2).shape, w.permute(0, 3, 1, 2),
                                         gout.permute(0, 3, 1, 2), padding=1).permute(0, 2, 3, 1)
        if mask is not None:
            gin = torch.where(mask > 0, gin, torch.zeros_like(gin))
        return bf(gin)

    def upbwd(gu, mask):
        g = ((gu[:, 0::2, 0::2] + gu[:, 0::2, 1::2]) + gu[:, 1::2, 0::2]) + gu[:, 1::2, 1::2]
        return bf(torch.where(mask > 0, g, torch.zeros_like(g)))

    def poolbwd(gp, add, mask):
        g = 0.25 * _up(gp) + add
        return bf(torch.where(mask > 0, g, torch.zeros_like(g)))

    g10 = back(11, a[10], gy, a[10])
    gu0 = back(10, a["u0"], g10, None)
    g9 = upbwd(gu0, a[9])
    gu1 = back(9, a["u1"], g9, None)
    g8 = upbwd(gu1, a[8])
    gu2 = back(8, a["u2"], g8, None)
    g7 = upbwd(gu2, a[7])
    g6 = back(7, a[6], g7, a[6])
    gp2 = back(6, a["p2"], g6, None)
    g5 = poolbwd(gp2, gu2, a[5])
    g4 = back(5, a[4], g5, a[4])
    gp1 = back(4, a["p1"], g4, None)
    g3 = poolbwd(gp1, gu1, a[3])
    g2 = back(3, a[2], g3, a[2])
    gp0 = back(2, a["p0"], g2, None)
    g1 = poolbwd(gp0, gu0, a[1])
    g0 = back(1, a[0], g1, a[0])
    back(0, a["x"], g0, None)
    flat = np.concatenate([np.concatenate([gw.reshape(-1).detach().numpy(), gb.detach().numpy()])
                           for gw, gb in grads])
    return loss, flat, y


def layer_slices():
    """(start, stop) of each layer's weights and bias in the flat vector."""
    out, o = [], 0
    for ci, co, _, _ in LAYERS:
        out.append(((o, o + co * 9 * ci), (o + co * 9 * ci, o + co * 9 * ci + co)))
        o += co * 9 * ci + co
    return out


# ---- inputs and outputs of the solver (jmg_net_inputs_2d / jmg_net_guess_2d) -------------

def inputs_2d(m, res, lam, dxx, dyy, rhs):
    """Packed input [res,res,16] (BF16 values, float32 array) and the pooled rhs RMS."""
    f = m // res
    full = lambda v: np.broadcast_to(np.asarray(v, dtype=np.float64), rhs.shape)
    blk = lambda v: full(v)[1:1 + f * res, 1:1 + f * res].reshape(res, f, res, f).mean(axis=(1, 3))
    c0, c1 = blk(np.log(full(dxx))), blk(np.log(full(dyy)))
    c2, c3 = blk(lam) * 0.1, blk(rhs)
    c3f = c3.astype(np.float32)
    rms = float(np.float32(np.sqrt(np.mean(c3f.astype(np.float64) ** 2))))
    if rms == 0:
        rms = 1.0
    x = np.zeros((res, res, 16), np.float32)
    x[..., 0], x[..., 1], x[..., 2] = c0.astype(np.float32), c1.astype(np.float32), c2.astype(np.float32)
    x[..., 3] = c3f * np.float32(1.0 / np.float32(rms))
    return bf(torch.from_numpy(x)).numpy(), rms


def output_2d(y, rms, out_scale, m):
    """phi0 [(m+3),(m+3)] from the network output y [res,res] (bilinear, zero frame)."""
    res = y.shape[0]
    f = m // res
    idx = np.arange(m + 3)
    u = (idx - 1 - 0.5 * (f - 1)) / f
    b0 = np.floor(u).astype(int)
    w = u - b0
    lo = b0 < 0
    b0[lo], w[lo] = 0, 0.0
    hi = b0 > res - 2
    w[hi] = np.minimum(u[hi] - (res - 2), 1.0)
    b0[hi] = res - 2
    y = y.astype(np.float64)
    rows = (1 - w)[None, :] * y[:, b0] + w[None, :] * y[:, b0 + 1]        # [res, m+3] along x
    phi = (1 - w)[:, None] * rows[b0, :] + w[:, None] * rows[b0 + 1, :]   # along y
    phi = phi * (float(out_scale) * float(rms))
    out = np.zeros((m + 3, m + 3))
    out[2:m + 1, 2:m + 1] = phi[2:m + 1, 2:m + 1]
    return out


def ritz_scale(g, rhs, lam, dxx, dyy, m):
    """beta = (g . rhs) / (g . L g) over the interior, L the 2D level-0 operator with face
    averages (the solver's), 0 when not positive (jmg_net_guess_2d's final scaling)."""
    full = lambda v: np.broadcast_to(np.asarray(v, dtype=np.float64), rhs.shape)
    Dx, Dy, lm = full(dxx), full(dyy), full(lam)
    s2 = float(m) ** 2
    i = slice(2, m + 1)
    ex = 0.5 * (Dx[i, 2:m + 1] + Dx[i, 3:m + 2]) * s2
    wx = 0.5 * (Dx[i, 1:m] + Dx[i, 2:m + 1]) * s2
    ny = 0.5 * (Dy[2:m + 1, i] + Dy[3:m + 2, i]) * s2
    sy = 0.5 * (Dy[1:m, i] + Dy[2:m + 1, i]) * s2
    cc = ex + wx + ny + sy + lm[i, i]
    lg = ex * g[i, 3:m + 2] + wx * g[i, 1:m] + ny * g[3:m + 2, i] + sy * g[1:m, i] - cc * g[i, i]
    a = float(np.sum(g[i, i] * rhs[i, i]))
    b = float(np.sum(g[i, i] * lg))
    return a / b if b != 0 and a / b > 0 else 0.0
