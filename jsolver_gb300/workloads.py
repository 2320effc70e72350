"""Seeded synthetic problems for benchmarks and tests (host NumPy, input generation only).

The reference publishes no dataset: its benchmark problems are analytic (see the
reference's examples/benchmark.py). The random-coefficient workloads here are the
ones this project is measured on:

* ``random_2d(m, seed)``: 2D m x m grid, arrays (m+3)^2 float64. D_xx, D_yy are
  independent log-normal fields exp(g), g a Gaussian random field with sigma = 1 and
  correlation length 0.05 (Gaussian covariance exp(-r^2 / (2 l^2))), synthesised
  spectrally on the periodic padded cell-centre grid. lambda ~ U[0, 10] i.i.d. per
  cell. rhs = L_h phi* for phi* = sin(pi x) sin(2 pi y) with the discrete level-0
  operator, so phi* (zero frame) is the exact discrete solution.
* ``random_3d(m, seed)``: 3D m^3 grid, arrays (m+3)^3. D_xx, D_yy, D_zz =
  exp(GRF sigma=1.2, l=0.08). lambda = exp(GRF) min-max scaled to [0, 50]. rhs =
  smooth GRF noise + a Gaussian source of width 0.02 at a seeded centre.

The level-0 operator used for the manufactured rhs follows the reference's
discretisation (2D: solver_2d.py:359-409 face averages; 3D: solver_3d.py:413-422 raw
cell values) and is applied on interior indices 2..m only.
"""
import numpy as np


def grf(shape, spacing, corr_len, sigma, rng):
    """Zero-mean Gaussian random field with Gaussian covariance, periodic, unit-normalised."""
    white = rng.standard_normal(shape)
    f = np.fft.rfftn(white)
    ks = [np.fft.fftfreq(n, d=spacing) * 2 * np.pi for n in shape[:-1]]
    ks.append(np.fft.rfftfreq(shape[-1], d=spacing) * 2 * np.pi)
    k2 = np.zeros(f.shape)
    for ax, k in enumerate(ks):
        sh = [1] * len(shape)
        sh[ax] = k.size
        k2 = k2 + (k.reshape(sh)) ** 2
    f *= np.exp(-0.25 * k2 * corr_len ** 2)  # sqrt of the Gaussian spectral density
    g = np.fft.irfftn(f, s=shape, axes=tuple(range(len(shape))))
    g -= g.mean()
    g /= g.std()
    return sigma * g


def centers(m, xb=0.0, xe=1.0):
    """Cell centres of a linear rim-1 grid (same as ``grid_1D(m).centers``)."""
    h = (xe - xb) / m
    return (np.arange(-1, m + 2) - 0.5 + 0.5) * h + xb


def apply_operator_2d(phi, Dxx, Dyy, lam, idel_x, idel_y):
    """L_h phi on interior indices 2..m (zero elsewhere), level-0 2D coefficients."""
    Dx = Dxx.copy()
    Dy = Dyy.copy()
    Dx[1:-1, :-1] = 0.5 * (Dxx[1:-1, 1:] + Dxx[1:-1, :-1])
    Dy[:-1, 1:-1] = 0.5 * (Dyy[1:, 1:-1] + Dyy[:-1, 1:-1])
    sx, sy = idel_x ** 2, idel_y ** 2
    out = np.zeros_like(phi)
    i = slice(2, -2)
    lc = Dx[i, 1:-3] * sx
    rc = Dx[i, 2:-2] * sx
    cl = Dy[1:-3, i] * sy
    cr = Dy[2:-2, i] * sy
    lamc = lam if np.ndim(lam) == 0 else lam[i, i]
    cc = lc + rc + cl + cr + lamc
    out[i, i] = (lc * phi[i, 1:-3] + rc * phi[i, 3:-1] + cl * phi[1:-3, i] + cr * phi[3:-1, i]
                 - cc * phi[i, i])
    return out


def apply_operator_3d(phi, Dxx, Dyy, Dzz, lam, idel):
    """L_h phi on interior indices 2..m, level-0 3D coefficients (raw cell values)."""
    sx, sy, sz = (d ** 2 for d in idel)
    out = np.zeros_like(phi)
    i = slice(2, -2)
    lcc = Dxx[i, i, 1:-3] * sx
    rcc = Dxx[i, i, i] * sx
    clc = Dyy[i, 1:-3, i] * sy
    crc = Dyy[i, i, i] * sy
    ccl = Dzz[1:-3, i, i] * sz
    ccr = Dzz[i, i, i] * sz
    lamc = lam if np.ndim(lam) == 0 else lam[i, i, i]
    ccc = lcc + rcc + clc + crc + ccl + ccr + lamc
    out[i, i, i] = (lcc * phi[i, i, 1:-3] + rcc * phi[i, i, 3:-1] + clc * phi[i, 1:-3, i]
                    + crc * phi[i, 3:-1, i] + ccl * phi[1:-3, i, i] + ccr * phi[3:-1, i, i]
                    - ccc * phi[i, i, i])
    return out


def _zero_frame(a):
    for ax in range(a.ndim):
        idx = [slice(None)] * a.ndim
        for s in (slice(0, 2), slice(-2, None)):
            idx[ax] = s
            a[tuple(idx)] = 0.0
    return a


def random_2d(m, seed=0, corr_len=0.05, sigma=1.0, lam_max=10.0):
    """2D random-coefficient problem. Returns dict(phi0, rhs, lam, D_xx, D_yy, phi_exact, m)."""
    rng = np.random.default_rng(seed)
    n = m + 3
    h = 1.0 / m
    Dxx = np.exp(grf((n, n), h, corr_len, sigma, rng))
    Dyy = np.exp(grf((n, n), h, corr_len, sigma, rng))
    lam = rng.uniform(0.0, lam_max, size=(n, n))
    c = centers(m)
    phi_exact = _zero_frame(np.sin(np.pi * c)[None, :] * np.sin(2 * np.pi * c)[:, None])
    rhs = apply_operator_2d(phi_exact, Dxx, Dyy, lam, float(m), float(m))
    return dict(m=m, phi0=np.zeros((n, n)), rhs=rhs, lam=lam, D_xx=Dxx, D_yy=Dyy, phi_exact=phi_exact)


def random_3d(m, seed=0, corr_len=0.08, sigma=1.2, lam_max=50.0, src_width=0.02):
    """3D random-coefficient problem. Returns dict(phi0, rhs, lam, D_xx, D_yy, D_zz, m)."""
    rng = np.random.default_rng(seed)
    n = m + 3
    h = 1.0 / m
    Ds = [np.exp(grf((n, n, n), h, corr_len, sigma, rng)) for _ in range(3)]
    g = np.exp(grf((n, n, n), h, corr_len, 1.0, rng))
    lam = lam_max * (g - g.min()) / (g.max() - g.min())
    noise = grf((n, n, n), h, corr_len, 1.0, rng)
    c = centers(m)
    x0 = rng.uniform(0.25, 0.75, size=3)
    r2 = ((c[None, None, :] - x0[0]) ** 2 + (c[None, :, None] - x0[1]) ** 2
          + (c[:, None, None] - x0[2]) ** 2)
    src = np.exp(-r2 / (2 * src_width ** 2)) / (2 * np.pi * src_width ** 2) ** 1.5
    rhs = _zero_frame(-(noise + src))
    return dict(m=m, phi0=np.zeros((n, n, n)), rhs=rhs, lam=lam, D_xx=Ds[0], D_yy=Ds[1], D_zz=Ds[2])
