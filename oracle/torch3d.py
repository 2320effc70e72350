"""CPU oracle (test infrastructure only): differentiable float64 torch restatement of the
reference's 3D solve, whose torch.func.jvp stands in for ``jax.jvp`` of ``solve_3d`` (the
reference checks forward mode on every 3D problem, tests/test_solver_3d.py:208-211; JAX is
not available to run the reference itself) and whose autograd stands in for ``jax.vjp``
of its fixed mode (solver_3d.py:468-470).

Same operations as ``oracle/mg3d.py`` (which is pinned to the reference's goldens),
written functionally so that torch records every step:
  * coefficient hierarchy, solver_3d.py:338-429: level 0 keeps the raw cell D, level
    l >= 1 injects level l-1 and face-averages; lambda is injected;
  * red-black Gauss-Seidel over the 8 sub-lattices in the reference's order, 679-706;
  * defect + restriction from the 12 edge-diagonal red neighbours, 622-652;
  * prolongation (trilinear points always, bilinear ones when nu2 <= 0), 654-677;
  * the cycle recursion, 588-620, and the fixed loop with skip_pre, 457-470.
Scalar D and lambda are taken as constant arrays (the same values; the reference's
scalar formulas differ from them only by rounding). Only the checkers of the CUDA
tangent and adjoint import it.
"""
import torch

from .mg3d import SUBLATTICES_3D, level_layout


def _frame0(a):
    a = a.clone()
    a[:, :, :2] = 0
    a[:, :, -2:] = 0
    a[:, :2] = 0
    a[:, -2:] = 0
    a[:2] = 0
    a[-2:] = 0
    return a


class Torch3D:
    def __init__(self, mx, my, mz, idel, gamma=1, fcycle=False, nu1=1, nu2=1, skip_pre=False):
        self.levels, self.mxl, self.myl, self.mzl, self.shapes = level_layout(mx, my, mz)
        L = self.levels
        self.idel = [[d * 0.5 ** l for l in range(L)] for d in idel]  # per axis x, y, z
        self.gamma, self.fcycle, self.nu1, self.nu2, self.skip_pre = gamma, fcycle, nu1, nu2, skip_pre

    def _inject(self, a, l):
        z = torch.zeros(self.shapes[l], dtype=torch.float64)
        z[1:-1, 1:-1, 1:-1] = a[1::2, 1::2, 1::2]
        return z

    def hierarchy(self, lam, Dxx, Dyy, Dzz):
        """Per-level (lcc, rcc, clc, crc, ccl, ccr, ccc) (solver_3d.py:338-429)."""
        L = self.levels
        shape0 = self.shapes[0]
        full = [x.expand(shape0) if x.dim() == 0 else x for x in (lam, Dxx, Dyy, Dzz)]
        lm, Dx, Dy, Dz = [full[0]], [full[1]], [full[2]], [full[3]]
        for l in range(1, L):
            lm.append(self._inject(lm[l - 1], l))
            nx_, ny_, nz_ = self._inject(Dx[l - 1], l), self._inject(Dy[l - 1], l), self._inject(Dz[l - 1], l)
            ax, ay, az = nx_.clone(), ny_.clone(), nz_.clone()
            ax[1:-1, 1:-1, :-1] = 0.5 * (nx_[1:-1, 1:-1, 1:] + nx_[1:-1, 1:-1, :-1])
            ay[1:-1, :-1, 1:-1] = 0.5 * (ny_[1:-1, 1:, 1:-1] + ny_[1:-1, :-1, 1:-1])
            az[:-1, 1:-1, 1:-1] = 0.5 * (nz_[1:, 1:-1, 1:-1] + nz_[:-1, 1:-1, 1:-1])
            Dx.append(ax)
            Dy.append(ay)
            Dz.append(az)
        out = []
        for l in range(L):
            sx, sy, sz = (self.idel[a][l] ** 2 for a in range(3))
            lcc = Dx[l][1:-1, 1:-1, 0:-2] * sx
            rcc = Dx[l][1:-1, 1:-1, 1:-1] * sx
            clc = Dy[l][1:-1, 0:-2, 1:-1] * sy
            crc = Dy[l][1:-1, 1:-1, 1:-1] * sy
            ccl = Dz[l][0:-2, 1:-1, 1:-1] * sz
            ccr = Dz[l][1:-1, 1:-1, 1:-1] * sz
            ccc = lcc + rcc + clc + crc + ccl + ccr + lm[l][1:-1, 1:-1, 1:-1]
            out.append((lcc, rcc, clc, crc, ccl, ccr, ccc))
        return out

    def rbgs(self, phi, rhs, A):
        lcc, rcc, clc, crc, ccl, ccr, ccc = A
        phi = _frame0(phi)
        for (lx, ly, lz) in SUBLATTICES_3D:
            P = phi
            t = (slice(lz + 1, -1, 2), slice(ly + 1, -1, 2), slice(lx + 1, -1, 2))
            c = (slice(lz, None, 2), slice(ly, None, 2), slice(lx, None, 2))
            U = P[lz + 2::2, ly + 1:-1:2, lx + 1:-1:2]
            D = P[lz:-2:2, ly + 1:-1:2, lx + 1:-1:2]
            N = P[lz + 1:-1:2, ly + 2::2, lx + 1:-1:2]
            S = P[lz + 1:-1:2, ly:-2:2, lx + 1:-1:2]
            E = P[lz + 1:-1:2, ly + 1:-1:2, lx + 2::2]
            W = P[lz + 1:-1:2, ly + 1:-1:2, lx:-2:2]
            new = (ccr[c] * U + ccl[c] * D + crc[c] * N + clc[c] * S + rcc[c] * E + lcc[c] * W - rhs[t]) / ccc[c]
            phi = phi.clone()
            phi[t] = new
            phi = _frame0(phi)
        return phi

    def defect(self, phi, rhs, A, level):
        lcc, rcc, clc, crc, ccl, ccr, ccc = A
        d = torch.zeros(rhs.shape, dtype=torch.float64)
        d[1:-1, 1:-1, 1:-1] = (ccc * phi[1:-1, 1:-1, 1:-1] - lcc * phi[1:-1, 1:-1, :-2] - rcc * phi[1:-1, 1:-1, 2:]
                               - clc * phi[1:-1, :-2, 1:-1] - crc * phi[1:-1, 2:, 1:-1] - ccl * phi[:-2, 1:-1, 1:-1]
                               - ccr * phi[2:, 1:-1, 1:-1] + rhs[1:-1, 1:-1, 1:-1])
        d = _frame0(d)
        r = torch.zeros(self.shapes[level + 1], dtype=torch.float64)
        r[1:-1, 1:-1, 1:-1] = 0.03125 * (
            d[1:-1:2, 2::2, 2::2] + d[1:-1:2, 2::2, :-2:2] + d[1:-1:2, :-2:2, 2::2] + d[1:-1:2, :-2:2, :-2:2]
            + d[2::2, 1:-1:2, 2::2] + d[2::2, 1:-1:2, :-2:2] + d[:-2:2, 1:-1:2, 2::2] + d[:-2:2, 1:-1:2, :-2:2]
            + d[2::2, 2::2, 1:-1:2] + d[2::2, :-2:2, 1:-1:2] + d[:-2:2, 2::2, 1:-1:2] + d[:-2:2, :-2:2, 1:-1:2]
        ) + 0.125 * d[1:-1:2, 1:-1:2, 1:-1:2]
        return _frame0(r)

    def prolongate(self, phi_c, level):
        c = torch.zeros(self.shapes[level], dtype=torch.float64)
        c[1:-1:2, 1:-1:2, 1:-1:2] = phi_c[1:-1, 1:-1, 1:-1]
        c[1:-1:2, 1:-1:2, 2:-1:2] = 0.5 * (c[1:-1:2, 1:-1:2, 3::2] + c[1:-1:2, 1:-1:2, 1:-2:2])
        c[1:-1:2, 2:-1:2, 1:-1:2] = 0.5 * (c[1:-1:2, 3::2, 1:-1:2] + c[1:-1:2, 1:-2:2, 1:-1:2])
        c[2:-1:2, 1:-1:2, 1:-1:2] = 0.5 * (c[3::2, 1:-1:2, 1:-1:2] + c[1:-2:2, 1:-1:2, 1:-1:2])
        if self.nu2 <= 0:
            c[1:-1:2, 2:-1:2, 2:-1:2] = 0.25 * (c[1:-1:2, 3::2, 3::2] + c[1:-1:2, 1:-2:2, 3::2]
                                               + c[1:-1:2, 3::2, 1:-2:2] + c[1:-1:2, 1:-2:2, 1:-2:2])
            c[2:-1:2, 1:-1:2, 2:-1:2] = 0.25 * (c[3::2, 1:-1:2, 3::2] + c[1:-2:2, 1:-1:2, 3::2]
                                               + c[3::2, 1:-1:2, 1:-2:2] + c[1:-2:2, 1:-1:2, 1:-2:2])
            c[2:-1:2, 2:-1:2, 1:-1:2] = 0.25 * (c[3::2, 3::2, 1:-1:2] + c[1:-2:2, 3::2, 1:-1:2]
                                               + c[3::2, 1:-2:2, 1:-1:2] + c[1:-2:2, 1:-2:2, 1:-1:2])
        c[2:-1:2, 2:-1:2, 2:-1:2] = 0.125 * (
            c[3::2, 3::2, 3::2] + c[1:-2:2, 3::2, 3::2] + c[3::2, 1:-2:2, 3::2] + c[1:-2:2, 1:-2:2, 3::2]
            + c[3::2, 3::2, 1:-2:2] + c[1:-2:2, 3::2, 1:-2:2] + c[3::2, 1:-2:2, 1:-2:2] + c[1:-2:2, 1:-2:2, 1:-2:2])
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

    def solve_fixed(self, phi0, rhs, lam, Dxx, Dyy, Dzz, iters):
        """solve_3d with a fixed count of cycles (solver_3d.py:457-470), differentiable in
        every input; with the primal's count it is also the dynamic solve's map."""
        H = self.hierarchy(lam, Dxx, Dyy, Dzz)
        phi = phi0
        if self.skip_pre:
            for _ in range(self.nu1):
                phi = self.rbgs(phi, rhs, H[0])
        for _ in range(iters):
            phi = self.cycle(_frame0(phi), rhs, H, self.fcycle, 0, self.skip_pre)
        return phi
