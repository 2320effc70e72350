"""CPU oracle (test infrastructure only): NumPy restatement of jsolver's 2D multigrid.

This module is the checker for the CUDA solver in ``jsolver_gb300``. It is not a
product path: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may import it.

It restates, operation for operation and in the same floating-point order,
``jsolver/solver_2d.py`` and ``jsolver/boundary_handler_2d.py`` of davef96/jsolver:

* levels / shapes ............ solver_2d.py:279-307 (``compute_shapes``)
* idel per level ............. solver_2d.py:309-324 (``compute_idel``)
* D face averaging ........... solver_2d.py:326-363 (``compute_diffusion_tensor``)
* lambda injection ........... solver_2d.py:365-383 (``compute_lambda``)
* stencil coefficients ....... solver_2d.py:385-421 (``compute_discretization``)
* driver (fixed/dynamic) ..... solver_2d.py:423-479 (``solve``)
* distance ................... solver_2d.py:481-494
* cycle recursion ............ solver_2d.py:582-614 (``multigrid_cycle``)
* defect + restriction ....... solver_2d.py:616-647 (``defect``)
* prolongation ............... solver_2d.py:649-668 (``prolongate``)
* red-black Gauss-Seidel ..... solver_2d.py:670-692
* boundary frame ............. boundary_handler_2d.py:3-30 (``do_BCs``)

Parity is pinned against the reference's own known-answer tests (iteration count +
RMSE against the analytic solution) in tests/test_solver_2d.py and the golden
dictionaries of examples/benchmark.py:26-632; see ``tests/test_oracle_goldens.py``.
"""
import numpy as np

INT32_MAX = int(np.iinfo(np.int32).max)


def do_bcs(arr, rim=1, direction=-1, vals_xb=None, vals_xe=None, vals_yb=None, vals_ye=None):
    """Zero (or set) the first/last ``rim+1`` columns then rows (boundary_handler_2d.py:3-30).

    Returns a new array; the input is not modified.
    """
    arr = np.array(arr, dtype=np.float64, copy=True)
    upper = rim + 1
    if direction in (-1, 0):
        arr[:, :upper] = 0 if vals_xb is None else np.asarray(vals_xb)[:, None]
        arr[:, -upper:] = 0 if vals_xe is None else np.asarray(vals_xe)[:, None]
    if direction in (-1, 1):
        arr[:upper] = 0 if vals_yb is None else np.asarray(vals_yb)[None, :]
        arr[-upper:] = 0 if vals_ye is None else np.asarray(vals_ye)[None, :]
    return arr


def _zero_frame(a):
    """In-place ``do_BCs`` with rim=1 (frame indices 0, 1, -2, -1 on both axes)."""
    a[:, :2] = 0.0
    a[:, -2:] = 0.0
    a[:2] = 0.0
    a[-2:] = 0.0
    return a


def _is_scalar(v):
    return np.ndim(v) == 0


def level_layout(mx, my):
    """Number of levels and per-level resolutions (solver_2d.py:279-307).

    Raises ValueError with the reference's messages, x before y, power-of-2 checks
    before efficiency checks.
    """
    if (mx & (mx - 1)) > 0:
        raise ValueError(f"Resolution of x-grid is not a power of 2. Value: {mx}")
    if (my & (my - 1)) > 0:
        raise ValueError(f"Resolution of y-grid is not a power of 2. Value: {my}")
    xl = int(np.ceil(np.log2(mx))) + 1
    yl = int(np.ceil(np.log2(my))) + 1
    levels = min(xl, yl)
    mxl = [2 ** (xl - 1 - l) for l in range(levels)]
    myl = [2 ** (yl - 1 - l) for l in range(levels)]
    if mxl[-1] > 5:
        raise ValueError(f"Resolution of x-grid not efficient for multigrid configuration. Resolution of coarsest level: {mxl[-1]}")
    if myl[-1] > 5:
        raise ValueError(f"Resolution of y-grid not efficient for multigrid configuration. Resolution of coarsest level: {myl[-1]}")
    shapes = [(myl[l] + 3, mxl[l] + 3) for l in range(levels)]
    return levels, mxl, myl, shapes


class Hierarchy2D:
    """Per-level stencil coefficients, built exactly as solver_2d.py:326-421.

    For spatially varying D, ``lc, rc, cl, cr, cc`` are (m_l+1)^2 arrays aligned with
    phi[1:-1, 1:-1] (left/right x-faces, lower/upper y-faces, centre). For scalar D,
    ``ax, ay`` are per-level scalars and ``cc`` is a scalar or an (m_l+1)^2 array.
    With D_xy, the diagonal couplings ``ll, lr, rl, rr`` are present as well.
    """

    def __init__(self, idel_x, idel_y, mx, my, lam, D_xx, D_yy, D_xy=None):
        self.levels, self.mxl, self.myl, self.shapes = level_layout(mx, my)
        L = self.levels
        self.idel_x = idel_x * 0.5 ** np.arange(L)
        self.idel_y = idel_y * 0.5 ** np.arange(L)
        self.scalar_lambda = _is_scalar(lam)
        self.spatial = not (_is_scalar(D_xx) and _is_scalar(D_yy))
        self.off_diag = self.spatial and D_xy is not None
        sqx = self.idel_x ** 2
        sqy = self.idel_y ** 2

        lam_l = None
        if not self.scalar_lambda:
            # compute_lambda, solver_2d.py:365-383: inject odd points, ring stays zero
            lam_l = [np.asarray(lam, dtype=np.float64)]
            for l in range(1, L):
                a = np.zeros(self.shapes[l])
                a[1:-1, 1:-1] = lam_l[l - 1][1::2, 1::2]
                lam_l.append(a)
        self.lam_levels = lam_l

        if self.spatial:
            # compute_diffusion_tensor, solver_2d.py:341-361: inject raw values to every
            # level first, then face-average every level (level 0 included)
            Dx = [np.array(D_xx, dtype=np.float64, copy=True)]
            Dy = [np.array(D_yy, dtype=np.float64, copy=True)]
            Dxy = [np.array(D_xy, dtype=np.float64, copy=True)] if self.off_diag else None
            for l in range(1, L):
                for lst in ([Dx, Dy] + ([Dxy] if self.off_diag else [])):
                    a = np.zeros(self.shapes[l])
                    a[1:-1, 1:-1] = lst[l - 1][1::2, 1::2]
                    lst.append(a)
            for l in range(L):
                Dx[l][1:-1, :-1] = 0.5 * (Dx[l][1:-1, 1:] + Dx[l][1:-1, :-1])
                Dy[l][:-1, 1:-1] = 0.5 * (Dy[l][1:, 1:-1] + Dy[l][:-1, 1:-1])
            self.Dx, self.Dy, self.Dxy = Dx, Dy, Dxy
            # compute_discretization, solver_2d.py:403-416
            self.lc = [Dx[l][1:-1, 0:-2] * sqx[l] for l in range(L)]
            self.rc = [Dx[l][1:-1, 1:-1] * sqx[l] for l in range(L)]
            self.cl = [Dy[l][0:-2, 1:-1] * sqy[l] for l in range(L)]
            self.cr = [Dy[l][1:-1, 1:-1] * sqy[l] for l in range(L)]
            self.cc = [self.lc[l] + self.rc[l] + self.cl[l] + self.cr[l]
                       + (lam if self.scalar_lambda else lam_l[l][1:-1, 1:-1]) for l in range(L)]
            if self.off_diag:
                cxy = self.idel_x * self.idel_y * 0.25
                self.ll = [(Dxy[l][1:-1, 0:-2] + Dxy[l][0:-2, 1:-1]) * cxy[l] for l in range(L)]
                self.lr = [-(Dxy[l][1:-1, 0:-2] + Dxy[l][2:, 1:-1]) * cxy[l] for l in range(L)]
                self.rl = [-(Dxy[l][1:-1, 2:] + Dxy[l][0:-2, 1:-1]) * cxy[l] for l in range(L)]
                self.rr = [(Dxy[l][1:-1, 2:] + Dxy[l][2:, 1:-1]) * cxy[l] for l in range(L)]
        else:
            # scalar diffusion, solver_2d.py:418-421
            self.ax = float(D_xx) * sqx
            self.ay = float(D_yy) * sqy
            add = 2 * (self.ax + self.ay)
            if self.scalar_lambda:
                self.cc = add + lam
            else:
                self.cc = [add[l] + lam_l[l][1:-1, 1:-1] for l in range(L)]

    def stencil(self, level):
        """Full-size (m_l+1)^2 coefficient arrays of one level (for kernels/tests)."""
        shp = (self.shapes[level][0] - 2, self.shapes[level][1] - 2)
        if self.spatial:
            out = dict(lc=self.lc[level], rc=self.rc[level], cl=self.cl[level],
                       cr=self.cr[level], cc=self.cc[level])
            if self.off_diag:
                out.update(ll=self.ll[level], lr=self.lr[level], rl=self.rl[level], rr=self.rr[level])
            return out
        ax, ay = self.ax[level], self.ay[level]
        cc = self.cc[level] if self.scalar_lambda else self.cc[level]
        return dict(lc=np.full(shp, ax), rc=np.full(shp, ax), cl=np.full(shp, ay),
                    cr=np.full(shp, ay), cc=np.broadcast_to(cc, shp).copy())


class Oracle2D:
    """The reference's Solver_2D restated (solver_2d.py:238-692)."""

    def __init__(self, grid_x, grid_y, fixed=False, epsilon=1e-12, gamma=1, fcycle=False,
                 skip_pre=False, nu1=1, nu2=1, max_iters_outer=INT32_MAX, max_iters_inner=INT32_MAX):
        self.fixed, self.epsilon, self.gamma, self.fcycle = fixed, epsilon, gamma, fcycle
        self.skip_pre, self.nu1, self.nu2 = skip_pre, nu1, nu2
        self.max_iters_outer, self.max_iters_inner = max_iters_outer, max_iters_inner
        self.levels, self.mxl, self.myl, self.shapes = level_layout(grid_x.mx, grid_y.mx)
        if not grid_x.is_linear or not grid_y.is_linear:
            raise ValueError("Only linear grids are supported!")
        self.grid_x, self.grid_y = grid_x, grid_y
        self.h = None

    # -- set-up -----------------------------------------------------------------
    def setup(self, phi, rhs, lam, D_xx, D_yy, D_xy=None):
        """dtype/shape checks (solver_2d.py:444-453) and coefficient hierarchy."""
        arrs = [phi, rhs, lam, D_xx, D_yy] + ([] if D_xy is None else [D_xy])
        if not all(np.asarray(a).dtype == np.float64 for a in arrs):
            raise ValueError("Incorrect configuration: dtype must be 'jnp.float64' for all arguments.")
        sl = _is_scalar(lam)
        spatial = not (_is_scalar(D_xx) and _is_scalar(D_yy))
        off = spatial and D_xy is not None
        s = np.shape
        if (not s(D_xx) == s(D_yy) or (sl and not s(phi) == s(rhs))
                or (not sl and not s(phi) == s(rhs) == s(lam))
                or (spatial and not s(phi) == s(rhs) == s(D_xx) == s(D_yy))
                or (off and not s(phi) == s(D_xy))
                or s(phi) != self.shapes[0]):
            raise ValueError(f"Shape mismatch: phi={s(phi)}, rhs={s(rhs)}, lam={s(lam)}, D_xx={s(D_xx)}, "
                             f"D_yy={s(D_yy)}, D_xy={'None' if D_xy is None else s(D_xy)}.")
        self.h = Hierarchy2D(self.grid_x.idel, self.grid_y.idel, self.grid_x.mx, self.grid_y.mx,
                             lam if sl else np.asarray(lam), D_xx, D_yy, D_xy)
        return self.h

    # -- operators --------------------------------------------------------------
    def rbgs(self, phi, rhs, level=0):
        """One red-black Gauss-Seidel sweep in place (solver_2d.py:670-692)."""
        h = self.h
        _zero_frame(phi)
        for (lx, ly) in ((0, 0), (1, 1), (0, 1), (1, 0)):
            P = phi
            sl_t = (slice(ly + 1, -1, 2), slice(lx + 1, -1, 2))
            N = P[ly + 2::2, lx + 1:-1:2]
            S = P[ly:-2:2, lx + 1:-1:2]
            E = P[ly + 1:-1:2, lx + 2::2]
            W = P[ly + 1:-1:2, lx:-2:2]
            r = rhs[sl_t]
            c = (slice(ly, None, 2), slice(lx, None, 2))
            if h.spatial:
                num = h.cr[level][c] * N + h.cl[level][c] * S + h.rc[level][c] * E + h.lc[level][c] * W - r
                if h.off_diag:
                    off = (h.ll[level][c] * P[ly:-2:2, lx:-2:2] + h.rl[level][c] * P[ly:-2:2, lx + 2::2]
                           + h.lr[level][c] * P[ly + 2::2, lx:-2:2] + h.rr[level][c] * P[ly + 2::2, lx + 2::2])
                    num = num + off
                new = num / h.cc[level][c]
            else:
                ax, ay = h.ax[level], h.ay[level]
                num = ay * N + ay * S + ax * E + ax * W - r
                new = num / (h.cc[level] if h.scalar_lambda else h.cc[level][c])
            phi[sl_t] = new
            _zero_frame(phi)
        return phi

    def defect_field(self, phi, rhs, level):
        """Fine-grid defect d = rhs - L_h phi with zero frame (solver_2d.py:632-642)."""
        h = self.h
        d = np.zeros(rhs.shape)
        C, W, E, S, N = phi[1:-1, 1:-1], phi[1:-1, :-2], phi[1:-1, 2:], phi[:-2, 1:-1], phi[2:, 1:-1]
        if h.spatial:
            off = 0
            if h.off_diag:
                off = (h.ll[level] * phi[:-2, :-2] + h.rl[level] * phi[:-2, 2:]
                       + h.lr[level] * phi[2:, :-2] + h.rr[level] * phi[2:, 2:])
            d[1:-1, 1:-1] = (h.cc[level] * C - h.lc[level] * W - h.rc[level] * E - h.cl[level] * S
                             - h.cr[level] * N + rhs[1:-1, 1:-1] - off)
        else:
            ax, ay = h.ax[level], h.ay[level]
            d[1:-1, 1:-1] = h.cc[level] * C - ax * W - ax * E - ay * S - ay * N + rhs[1:-1, 1:-1]
        return _zero_frame(d)

    def defect(self, phi, rhs, level):
        """Defect + red-point full weighting onto level+1 (solver_2d.py:616-647)."""
        d = self.defect_field(phi, rhs, level)
        rc = np.zeros(self.shapes[level + 1])
        rc[1:-1, 1:-1] = (0.0625 * (d[2::2, 2::2] + d[2::2, :-2:2] + d[:-2:2, 2::2] + d[:-2:2, :-2:2])
                          + 0.25 * d[1:-1:2, 1:-1:2])
        return _zero_frame(rc)

    def prolongate(self, phi_c, level):
        """Linear prolongation of the coarse correction (solver_2d.py:649-668)."""
        corr = np.zeros(self.shapes[level])
        corr[1:-1:2, 1:-1:2] = phi_c[1:-1, 1:-1]
        corr[1:-1:2, 2:-1:2] = 0.5 * (corr[1:-1:2, 3::2] + corr[1:-1:2, 1:-2:2])
        corr[2:-1:2, 1:-1:2] = 0.5 * (corr[3::2, 1:-1:2] + corr[1:-2:2, 1:-1:2])
        if self.nu2 <= 0 or self.h.off_diag:
            corr[2:-1:2, 2:-1:2] = 0.25 * (corr[3::2, 3::2] + corr[1:-2:2, 3::2]
                                           + corr[3::2, 1:-2:2] + corr[1:-2:2, 1:-2:2])
        return corr

    def cycle(self, phi, rhs, fcycle=False, level=0, skip_pre=False):
        """Recursive V/W/F cycle (solver_2d.py:582-614). Works in place on ``phi``."""
        if level == self.levels - 2:
            for _ in range(self.nu1 + self.nu2):
                self.rbgs(phi, rhs, level)
            return phi
        if not skip_pre:
            for _ in range(self.nu1):
                self.rbgs(phi, rhs, level)
        rhs_c = self.defect(phi, rhs, level)
        phi_c = np.zeros(self.shapes[level + 1])
        if fcycle:
            for _ in range(self.gamma):
                self.cycle(phi_c, rhs_c, True, level + 1)
        for _ in range(self.gamma):
            self.cycle(phi_c, rhs_c, False, level + 1)
        phi += self.prolongate(phi_c, level)
        for _ in range(self.nu2):
            self.rbgs(phi, rhs, level)
        return phi

    def solve(self, phi, rhs, lam, D_xx, D_yy, D_xy=None, callback=None):
        """Fixed or dynamic driver (solver_2d.py:423-479). Returns (phi, count)."""
        self.setup(phi, rhs, lam, D_xx, D_yy, D_xy)
        phi = np.array(phi, dtype=np.float64, copy=True)
        rhs = np.asarray(rhs, dtype=np.float64)
        if self.skip_pre:
            for _ in range(self.nu1):
                self.rbgs(phi, rhs, 0)
        if self.fixed:
            for it in range(self.max_iters_outer):
                _zero_frame(phi)
                self.cycle(phi, rhs, fcycle=self.fcycle, skip_pre=self.skip_pre)
                if callback is not None:
                    callback(it + 1, phi)
            return phi, self.max_iters_outer
        count, dist = 0, np.inf
        while dist > self.epsilon and count < self.max_iters_outer:
            phi_old = phi.copy()
            _zero_frame(phi)
            self.cycle(phi, rhs, fcycle=self.fcycle, skip_pre=self.skip_pre)
            dist = np.max(np.abs(phi_old - phi))
            count += 1
            if callback is not None:
                callback(count, phi)
        return phi, count

    # -- measurement helper (not in the reference solve path) --------------------
    def rel_residual(self, phi, rhs):
        """||rhs - L_h phi||_2 / ||rhs||_2 over the interior indices 2..m (FP64)."""
        d = self.defect_field(phi, rhs, 0)
        num = np.sqrt(np.sum(d[2:-2, 2:-2] ** 2))
        den = np.sqrt(np.sum(np.asarray(rhs)[2:-2, 2:-2] ** 2))
        return num / den


def solve_2d(grid_x, grid_y, phi, rhs, lam, D_xx, D_yy, *, D_xy=None, fixed=False, epsilon=1e-12,
             gamma=1, fcycle=False, skip_pre=False, nu1=1, nu2=1, max_iters_outer=INT32_MAX,
             max_iters_inner=INT32_MAX):
    """Oracle counterpart of ``solve_2d`` (solver_2d.py:196-236)."""
    o = Oracle2D(grid_x, grid_y, fixed=fixed, epsilon=epsilon, gamma=gamma, fcycle=fcycle,
                 skip_pre=skip_pre, nu1=nu1, nu2=nu2, max_iters_outer=max_iters_outer,
                 max_iters_inner=max_iters_inner)
    return o.solve(phi, rhs, lam, D_xx, D_yy, D_xy)
