"""CPU oracle (test infrastructure only): differentiable float64 torch restatement of the
reference's fixed-mode 2D solve, whose autograd stands in for ``jax.vjp`` of
``solve_2d_fixed_simple`` (the reference's reverse-mode path, jsolver/solver_2d.py:18-26,
tests/test_solver_2d.py:200-207; JAX is not available to run the reference itself) and
whose torch.func.jvp stands in for ``jax.jvp`` of the solve (tests/test_solver_2d.py:173-176;
with the primal's cycle count it is also the dynamic loop's map).

Same operations as ``oracle/mg2d.py`` (which is pinned to the reference's goldens), written
functionally so that torch records every step: coefficient hierarchy (solver_2d.py:326-421),
red-black Gauss-Seidel (670-692), defect + restriction (616-647), prolongation (649-668) and
the cycle recursion (582-614) with spatially varying D and lambda, the off-diagonal D_xy
terms of the 9-point stencil (345-349, 410-416, 636-641, 665-666, 686-690) and skip_pre
(457-459). Scalar D and lambda are taken as constant arrays (the same values; the
reference's scalar formulas differ from them only by rounding). Only the checkers of the
CUDA adjoint and tangent import it.
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
    def __init__(self, mx, my, idel_x, idel_y, gamma=1, fcycle=False, nu1=1, nu2=1, skip_pre=False):
        self.levels, self.mxl, self.myl, self.shapes = level_layout(mx, my)
        L = self.levels
        self.idel_x = [idel_x * 0.5 ** l for l in range(L)]
        self.idel_y = [idel_y * 0.5 ** l for l in range(L)]
        self.gamma, self.fcycle, self.nu1, self.nu2, self.skip_pre = gamma, fcycle, nu1, nu2, skip_pre
        self.off_diag = False

    def hierarchy(self, lam, Dxx, Dyy, Dxy=None):
        """Per-level (lc, rc, cl, cr, cc[, ll, lr, rl, rr]) as differentiable functions of
        lam, D (and D_xy) (solver_2d.py:341-416)."""
        L = self.levels
        shape0 = self.shapes[0]
        lam, Dxx, Dyy = (x.expand(shape0) if x.dim() == 0 else x for x in (lam, Dxx, Dyy))
        Dx, Dy, lm = [Dxx], [Dyy], [lam]
        Dxy_l = [Dxy] if Dxy is not None else None
        self.off_diag = Dxy is not None
        for l in range(1, L):
            for lst in (Dx, Dy, lm) + ((Dxy_l,) if Dxy_l is not None else ()):
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
            if Dxy_l is None:
                out.append((lc, rc, cl, cr, cc))
                continue
            cxy = self.idel_x[l] * self.idel_y[l] * 0.25
            X = Dxy_l[l]
            ll = (X[1:-1, 0:-2] + X[0:-2, 1:-1]) * cxy
            lr = -(X[1:-1, 0:-2] + X[2:, 1:-1]) * cxy
            rl = -(X[1:-1, 2:] + X[0:-2, 1:-1]) * cxy
            rr = (X[1:-1, 2:] + X[2:, 1:-1]) * cxy
            out.append((lc, rc, cl, cr, cc, ll, lr, rl, rr))
        return out

    def rbgs(self, phi, rhs, A):
        lc, rc, cl, cr, cc = A[:5]
        phi = _frame0(phi)
        for (lx, ly) in ((0, 0), (1, 1), (0, 1), (1, 0)):
            c = (slice(ly, None, 2), slice(lx, None, 2))
            num = (cr[c] * phi[ly + 2::2, lx + 1:-1:2] + cl[c] * phi[ly:-2:2, lx + 1:-1:2]
                   + rc[c] * phi[ly + 1:-1:2, lx + 2::2] + lc[c] * phi[ly + 1:-1:2, lx:-2:2]
                   - rhs[ly + 1:-1:2, lx + 1:-1:2])
            if len(A) > 5:
                ll, lr, rl, rr = A[5:]
                num = num + (ll[c] * phi[ly:-2:2, lx:-2:2] + rl[c] * phi[ly:-2:2, lx + 2::2]
                             + lr[c] * phi[ly + 2::2, lx:-2:2] + rr[c] * phi[ly + 2::2, lx + 2::2])
            new = num / cc[c]
            phi = phi.clone()
            phi[ly + 1:-1:2, lx + 1:-1:2] = new
            phi = _frame0(phi)
        return phi

    def defect(self, phi, rhs, A, level):
        lc, rc, cl, cr, cc = A[:5]
        d = torch.zeros(rhs.shape, dtype=torch.float64)
        off = 0
        if len(A) > 5:
            ll, lr, rl, rr = A[5:]
            off = ll * phi[:-2, :-2] + rl * phi[:-2, 2:] + lr * phi[2:, :-2] + rr * phi[2:, 2:]
        d[1:-1, 1:-1] = (cc * phi[1:-1, 1:-1] - lc * phi[1:-1, :-2] - rc * phi[1:-1, 2:] - cl * phi[:-2, 1:-1]
                         - cr * phi[2:, 1:-1] + rhs[1:-1, 1:-1] - off)
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
        if self.nu2 <= 0 or self.off_diag:
            c[2:-1:2, 2:-1:2] = 0.25 * (c[3::2, 3::2] + c[1:-2:2, 3::2] + c[3::2, 1:-2:2] + c[1:-2:2, 1:-2:2])
        return c

    def cycle(self, phi, rhs, H, fcycle=False, level=0, skip_pre=False):
        if level == self.levels - 2:
            for _ in range(self.nu1 + self.nu2):
                phi = self.rbgs(phi, rhs, H[level])
            return phi
        if not skip_pre:
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

    def solve_fixed(self, phi0, rhs, lam, Dxx, Dyy, iters, Dxy=None):
        """solve_2d in fixed mode (solver_2d.py:457-463), differentiable in every input;
        with the primal's count it is also the dynamic solve's map."""
        H = self.hierarchy(lam, Dxx, Dyy, Dxy)
        phi = phi0
        if self.skip_pre:
            for _ in range(self.nu1):
                phi = self.rbgs(phi, rhs, H[0])
        for _ in range(iters):
            phi = self.cycle(_frame0(phi), rhs, H, self.fcycle, 0, self.skip_pre)
        return phi
