"""CPU oracle (test infrastructure only): differentiable float64 torch restatement of the
reference's fixed-mode 2D solve, whose autograd stands in for ``jax.vjp`` of
``solve_2d_fixed_simple`` (the reference's reverse-mode path, jsolver/solver_2d.py:18-26,
tests/test_solver_2d.py:200-207; JAX is not available to run the reference itself).

Same operations as ``oracle/mg2d.py`` (which is pinned to the reference's goldens), written
functionally so that torch records every step: coefficient hierarchy (solver_2d.py:326-421),
red-black Gauss-Seidel (670-692), defect + restriction (616-647), prolongation (649-668) and
the cycle recursion (582-614) with spatially varying D and lambda. Only the checker of the
CUDA adjoint imports it.
"""
import torch

from .mg2d import level_layout


def _frame0(a):
    a = a.clone()
    a[:, :2] = 0
    a[:, -2:] = 0
    a[:2] = 0
    a[-2:] = 0
    return a


class Torch2D:
    def __init__(self, mx, my, idel_x, idel_y, gamma=1, fcycle=False, nu1=1, nu2=1):
        self.levels, self.mxl, self.myl, self.shapes = level_layout(mx, my)
        L = self.levels
        self.idel_x = [idel_x * 0.5 ** l for l in range(L)]
        self.idel_y = [idel_y * 0.5 ** l for l in range(L)]
        self.gamma, self.fcycle, self.nu1, self.nu2 = gamma, fcycle, nu1, nu2

    def hierarchy(self, lam, Dxx, Dyy):
        """Per-level (lc, rc, cl, cr, cc) as differentiable functions of lam, D (solver_2d.py:341-409)."""
        L = self.levels
        Dx, Dy, lm = [Dxx], [Dyy], [lam]
        for l in range(1, L):
            for lst in (Dx, Dy, lm):
                z = torch.zeros(self.shapes[l], dtype=torch.float64)
                z[1:-1, 1:-1] = lst[l - 1][1::2, 1::2]
                lst.append(z)
        out = []
        for l in range(L):
            sx, sy = self.idel_x[l] ** 2, self.idel_y[l] ** 2
            dx, dy = Dx[l].clone(), Dy[l].clone()
            dx[1:-1, :-1] = 0.5 * (Dx[l][1:-1, 1:] + Dx[l][1:-1, :-1])
            dy[:-1, 1:-1] = 0.5 * (Dy[l][1:, 1:-1] + Dy[l][:-1, 1:-1])
            lc = dx[1:-1, 0:-2] * sx
            rc = dx[1:-1, 1:-1] * sx
            cl = dy[0:-2, 1:-1] * sy
            cr = dy[1:-1, 1:-1] * sy
            cc = lc + rc + cl + cr + lm[l][1:-1, 1:-1]
            out.append((lc, rc, cl, cr, cc))
        return out

    def rbgs(self, phi, rhs, A):
        lc, rc, cl, cr, cc = A
        phi = _frame0(phi)
        for (lx, ly) in ((0, 0), (1, 1), (0, 1), (1, 0)):
            c = (slice(ly, None, 2), slice(lx, None, 2))
            new = (cr[c] * phi[ly + 2::2, lx + 1:-1:2] + cl[c] * phi[ly:-2:2, lx + 1:-1:2]
                   + rc[c] * phi[ly + 1:-1:2, lx + 2::2] + lc[c] * phi[ly + 1:-1:2, lx:-2:2]
                   - rhs[ly + 1:-1:2, lx + 1:-1:2]) / cc[c]
            phi = phi.clone()
            phi[ly + 1:-1:2, lx + 1:-1:2] = new
            phi = _frame0(phi)
        return phi

    def defect(self, phi, rhs, A, level):
        lc, rc, cl, cr, cc = A
        d = torch.zeros(rhs.shape, dtype=torch.float64)
        d[1:-1, 1:-1] = (cc * phi[1:-1, 1:-1] - lc * phi[1:-1, :-2] - rc * phi[1:-1, 2:] - cl * phi[:-2, 1:-1]
                         - cr * phi[2:, 1:-1] + rhs[1:-1, 1:-1])
        d = _frame0(d)
        r = torch.zeros(self.shapes[level + 1], dtype=torch.float64)
        r[1:-1, 1:-1] = (0.0625 * (d[2::2, 2::2] + d[2::2, :-2:2] + d[:-2:2, 2::2] + d[:-2:2, :-2:2])
                         + 0.25 * d[1:-1:2, 1:-1:2])
        return _frame0(r)

    def prolongate(self, phi_c, level):
        c = torch.zeros(self.shapes[level], dtype=torch.float64)
        c[1:-1:2, 1:-1:2] = phi_c[1:-1, 1:-1]
        c[1:-1:2, 2:-1:2] = 0.5 * (c[1:-1:2, 3::2] + c[1:-1:2, 1:-2:2])
        c[2:-1:2, 1:-1:2] = 0.5 * (c[3::2, 1:-1:2] + c[1:-2:2, 1:-1:2])
        if self.nu2 <= 0:
            c[2:-1:2, 2:-1:2] = 0.25 * (c[3::2, 3::2] + c[1:-2:2, 3::2] + c[3::2, 1:-2:2] + c[1:-2:2, 1:-2:2])
        return c

    def cycle(self, phi, rhs, H, fcycle=False, level=0):
        if level == self.levels - 2:
            for _ in range(self.nu1 + self.nu2):
                phi = self.rbgs(phi, rhs, H[level])
            return phi
        for _ in range(self.nu1):
            phi = self.rbgs(phi, rhs, H[level])
        rc = self.defect(phi, rhs, H[level], level)
        pc = torch.zeros(self.shapes[level + 1], dtype=torch.float64)
        if fcycle:
            for _ in range(self.gamma):
                pc = self.cycle(pc, rc, H, True, level + 1)
        for _ in range(self.gamma):
            pc = self.cycle(pc, rc, H, False, level + 1)
        phi = phi + self.prolongate(pc, level)
        for _ in range(self.nu2):
            phi = self.rbgs(phi, rhs, H[level])
        return phi

    def solve_fixed(self, phi0, rhs, lam, Dxx, Dyy, iters):
        """solve_2d in fixed mode (solver_2d.py:461-463), differentiable in every input."""
        H = self.hierarchy(lam, Dxx, Dyy)
        phi = phi0
        for _ in range(iters):
            phi = self.cycle(_frame0(phi), rhs, H, self.fcycle)
        return phi
