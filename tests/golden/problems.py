"""Manufactured problems of the reference's known-answer tests, restated.

Each builder returns ``(phi_exact, rhs, lam, D_xx, D_yy[, D_xy])`` (2D) or
``(phi_exact, rhs, lam, D_xx, D_yy, D_zz)`` (3D) on grid cell centres, following the
formulas of davef96/jsolver tests/test_solver_2d.py and tests/test_solver_3d.py (line
numbers beside each builder). Used with ``reference_goldens.json`` to pin the oracle
and the CUDA solver to the reference's iteration counts and RMSE values.
"""
import numpy as np

PI = np.pi


def p2d_1(xc, yc, shape):  # test_solver_2d.py:131-144
    x, y = xc[None], yc[:, None]
    ox, oy = 1. - x, 1. - y
    px3, py = x * ox ** 3, y * oy
    return px3 * py, -2 * px3 - 6 * ox * (ox - x) * py, 0.0, 1.0, 1.0


def p2d_2(xc, yc, shape):  # test_solver_2d.py:243-252
    sy, sx = np.sin(PI * yc)[:, None], np.sin(PI * xc)[None]
    phi = sx * sy
    return phi, -(PI ** 2) * (1.0 + 1.0) * phi, 0.0, 1.0, 1.0


def p2d_3(xc, yc, shape):  # test_solver_2d.py:321-332
    sy = np.sin(PI * yc)[:, None]
    x = xc[None]
    sx, cx = np.sin(PI * x), np.cos(PI * x)
    phi = sx * sy
    return phi, PI * cx * sy - 2 * PI ** 2 * x * phi, 0.0, np.full(shape, x), np.full(shape, x)


def p2d_4(xc, yc, shape):  # test_solver_2d.py:400-413
    y, x = yc[:, None], xc[None]
    sy, sx = np.sin(PI * y), np.sin(PI * x)
    phi = sx * sy
    lam = 0.2 * x * y ** 2
    s = x + y
    rhs = PI * np.sin(PI * s) - (s * PI ** 2 + lam) * phi
    return phi, rhs, lam, np.full(shape, x), np.zeros(shape) + y


def p2d_5(xc, yc, shape):  # test_solver_2d.py:479-490
    x, y = xc[None], yc[:, None]
    phi = np.sin(PI * x) * np.sin(PI * y)
    lam = 0.2 * x * y ** 2
    return phi, -((PI ** 2) * (1.0 + 1e-2) + lam) * phi, lam, 1.0, 1e-2


def _trig(xc, yc):
    y, x = yc[:, None], xc[None]
    return x, y, np.sin(PI * x), np.cos(PI * x), np.sin(PI * y), np.cos(PI * y)


def p2d_7(xc, yc, shape):  # test_solver_2d.py:558-573
    c = 0.1
    x, y, sx, cx, sy, cy = _trig(xc, yc)
    phi = sx * sy
    lam = 0.2 * x * y ** 2
    rhs = ((1. + c) * PI * sx * cy + PI * cx * sy + c * 2. * x * PI ** 2 * cx * cy
           - ((x + y) * PI ** 2 + lam) * phi)
    return phi, rhs, lam, np.full(shape, x), np.zeros(shape) + y, np.full(shape, c * x)


def p2d_9(xc, yc, shape):  # test_solver_2d.py:641-656
    c = 0.5
    x, y, sx, cx, sy, cy = _trig(xc, yc)
    phi = sx * sy
    lam = 0.2 * x * y ** 2
    rhs = ((1 + c * x) * PI * cx * sy + (1 + c * y) * PI * sx * cy + c * 2 * x * y * PI ** 2 * cx * cy
           - ((x + y) * PI ** 2 + lam) * phi)
    return phi, rhs, lam, np.full(shape, x), np.zeros(shape) + y, c * x * y


def p2d_10(xc, yc, shape):  # test_solver_2d.py:724-739
    c = 0.1
    x, y, sx, cx, sy, cy = _trig(xc, yc)
    phi = sx * sy
    lam = 0.2 * x * y ** 2
    rhs = (PI * (1 + c * y) * sx * cy + c * x * PI * cx * sy + c * 2 * x * y * PI ** 2 * cx * cy
           - (2 * y * PI ** 2 + lam) * phi)
    return phi, rhs, lam, np.zeros(shape) + y, np.zeros(shape) + y, c * x * y


def p2d_11(xc, yc, shape):  # test_solver_2d.py:807-836
    dpar, dperp = 1., 0.1
    x, y, sx, cx, sy, cy = _trig(xc, yc)
    phi = sx * sy
    lam = 0.2 * x * y ** 2
    ang = np.arctan2(y, x)
    sa, ca = np.sin(ang), np.cos(ang)
    sca, s2, c2 = sa * ca, sa ** 2, ca ** 2
    Dxx = dpar * s2 + dperp * c2
    Dyy = dpar * c2 + dperp * s2
    Dxy = (dperp - dpar) * sca
    r2 = x ** 2 + y ** 2
    with np.errstate(divide="ignore", invalid="ignore"):  # r2 = 0 at the origin, as defined
        dpx, dpy = -y / r2, x / r2
    dDxx_dx = 2 * (dpar - dperp) * sca * dpx
    dDyy_dy = 2 * (dperp - dpar) * sca * dpy
    dDxy_dx = (dperp - dpar) * (c2 - s2) * dpx
    dDxy_dy = (dperp - dpar) * (c2 - s2) * dpy
    rhs = ((dDyy_dy + dDxy_dx) * PI * sx * cy + (dDxx_dx + dDxy_dy) * PI * cx * sy
           + 2 * Dxy * PI ** 2 * cx * cy - ((Dxx + Dyy) * PI ** 2 + lam) * phi)
    return phi, rhs, lam, Dxx, Dyy, Dxy


PROBLEMS_2D = {1: p2d_1, 2: p2d_2, 3: p2d_3, 4: p2d_4, 5: p2d_5, 7: p2d_7, 9: p2d_9, 10: p2d_10, 11: p2d_11}


def _xyz(xc, yc, zc):
    return xc[None, None, :], yc[None, :, None], zc[:, None, None]


def p3d_1(xc, yc, zc):  # test_solver_3d.py:168-179
    x, y, z = _xyz(xc, yc, zc)
    phi = np.sin(PI * x) * np.sin(PI * y) * np.sin(PI * z)
    return phi, -(PI ** 2) * 3.0 * phi, 0.0, 1.0, 1.0, 1.0


def p3d_2(xc, yc, zc):  # test_solver_3d.py:248-262
    x, y, z = _xyz(xc, yc, zc)
    phi = np.sin(PI * x) * np.sin(PI * y) * np.sin(PI * z)
    lam = 0.2 * x * y ** 2 * z ** 3
    return phi, -((PI ** 2) * 3.0 + lam) * phi, lam, 1.0, 1.0, 1.0


def p3d_3(xc, yc, zc):  # test_solver_3d.py:330-344
    x, y, z = _xyz(xc, yc, zc)
    phi = np.sin(PI * x) * np.sin(PI * y) * np.sin(PI * z)
    lam = 0.2 * x * y ** 2 * z ** 3
    return phi, -((PI ** 2) * (1.0 + 0.5 + 2.0) + lam) * phi, lam, 1.0, 0.5, 2.0


PROBLEMS_3D = {1: p3d_1, 2: p3d_2, 3: p3d_3}


def rmse(phi_exact, phi):
    """Interior RMSE over indices 1..m+1 (test_solver_2d.py:20-23; test_solver_3d.py:19-22)."""
    sl = tuple(slice(1, -1) for _ in range(np.ndim(phi)))
    e = (phi_exact - phi)[sl]
    return float(np.linalg.norm(e.ravel()) / np.sqrt(e.size))


def make_2d(pid, mx, my, grid_cls):
    gx, gy = grid_cls(mx), grid_cls(my)
    shape = (my + 3, mx + 3)
    out = PROBLEMS_2D[pid](gx.centers, gy.centers, shape)
    phi_exact, rhs, lam = out[0], out[1], out[2]
    D = out[3:]
    return gx, gy, shape, phi_exact, np.broadcast_to(rhs, shape).copy(), lam, D


def make_3d(pid, mx, my, mz, grid_cls):
    gx, gy, gz = grid_cls(mx), grid_cls(my), grid_cls(mz)
    shape = (mz + 3, my + 3, mx + 3)
    phi_exact, rhs, lam, Dxx, Dyy, Dzz = PROBLEMS_3D[pid](gx.centers, gy.centers, gz.centers)
    if np.ndim(lam) > 0:
        lam = np.broadcast_to(lam, shape).copy()
    return gx, gy, gz, shape, np.broadcast_to(phi_exact, shape), np.broadcast_to(rhs, shape).copy(), lam, (Dxx, Dyy, Dzz)
