"""CPU oracle (test infrastructure only): NumPy restatement of jsolver's 3D multigrid.

Checker for the CUDA solver in ``jsolver_gb300``; never a product path. Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.

Restates ``jsolver/solver_3d.py`` and ``jsolver/boundary_handler_3d.py`` of
davef96/jsolver operation for operation:

* levels / shapes ............ solver_3d.py:281-317
* idel per level ............. solver_3d.py:319-336
* D hierarchy ................ solver_3d.py:338-372. Unlike 2D, level 0 keeps the raw
  cell values (the i<->i+1 coupling uses D[i]); level l>=1 injects from level l-1
  (already averaged for l-1>=1) and is then face-averaged.
* lambda injection ........... solver_3d.py:374-392
* stencil coefficients ....... solver_3d.py:394-429
* driver ..................... solver_3d.py:431-486
* cycle recursion ............ solver_3d.py:588-620
* defect + restriction ....... solver_3d.py:622-652 (12 edge-diagonal red neighbours)
* prolongation ............... solver_3d.py:654-677 (trilinear points always)
* red-black Gauss-Seidel ..... solver_3d.py:679-706 (8 sub-lattices)
* boundary frame ............. boundary_handler_3d.py:3-35

Pinned against tests/test_solver_3d.py of the reference (see tests/test_oracle_goldens.py).
"""
import numpy as np

INT32_MAX = int(np.iinfo(np.int32).max)

# sub-lattice order of the reference sweep (solver_3d.py:693), as (lx, ly, lz)
SUBLATTICES_3D = ((0, 0, 0), (0, 1, 1), (1, 1, 0), (1, 0, 1), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1))


def do_bcs(arr, rim=1, direction=-1, vals_xb=None, vals_xe=None, vals_yb=None, vals_ye=None,
           vals_zb=None, vals_ze=None):
    """boundary_handler_3d.py:3-35, including its use of ``vals_yb/vals_ye`` for the
    z faces (lines 32-33 of that file). Returns a new array."""
    arr = np.array(arr, dtype=np.float64, copy=True)
    upper = rim + 1
    if direction in (-1, 0):
        arr[:, :, :upper] = 0 if vals_xb is None else np.asarray(vals_xb)[:, :, None]
        arr[:, :, -upper:] = 0 if vals_xe is None else np.asarray(vals_xe)[:, :, None]
    if direction in (-1, 1):
        arr[:, :upper, :] = 0 if vals_yb is None else np.asarray(vals_yb)[:, None, :]
        arr[:, -upper:, :] = 0 if vals_ye is None else np.asarray(vals_ye)[:, None, :]
    if direction in (-1, 2):
        arr[:upper, :, :] = 0 if vals_yb is None else np.asarray(vals_yb)[None, :, :]
        arr[-upper:, :, :] = 0 if vals_ye is None else np.asarray(vals_ye)[None, :, :]
    return arr


def _zero_frame(a):
    a[:, :, :2] = 0.0
    a[:, :, -2:] = 0.0
    a[:, :2, :] = 0.0
    a[:, -2:, :] = 0.0
    a[:2] = 0.0
    a[-2:] = 0.0
    return a


def _is_scalar(v):
    return np.ndim(v) == 0


def level_layout(mx, my, mz):
    """solver_3d.py:281-317 (x, y, z order of the checks)."""
    for name, m in (("x", mx), ("y", my), ("z", mz)):
        if (m & (m - 1)) > 0:
            raise ValueError(f"Resolution of {name}-grid is not a power of 2. Value: {m}")
    xl = int(np.ceil(np.log2(mx))) + 1
    yl = int(np.ceil(np.log2(my))) + 1
    zl = int(np.ceil(np.log2(mz))) + 1
    levels = min(xl, yl, zl)
    mxl = [2 ** (xl - 1 - l) for l in range(levels)]
    myl = [2 ** (yl - 1 - l) for l in range(levels)]
    mzl = [2 ** (zl - 1 - l) for l in range(levels)]
    for name, ml in (("x", mxl), ("y", myl), ("z", mzl)):
        if ml[-1] > 5:
            raise ValueError(f"Resolution of {name}-grid not efficient for multigrid configuration. Resolution of coarsest level: {ml[-1]}")
    shapes = [(mzl[l] + 3, myl[l] + 3, mxl[l] + 3) for l in range(levels)]
    return levels, mxl, myl, mzl, shapes


class Hierarchy3D:
    """Per-level 7-point coefficients exactly as solver_3d.py:338-429."""

    def __init__(self, idel_x, idel_y, idel_z, mx, my, mz, lam, D_xx, D_yy, D_zz):
        self.levels, self.mxl, self.myl, self.mzl, self.shapes = level_layout(mx, my, mz)
        L = self.levels
        self.idel_x = idel_x * 0.5 ** np.arange(L)
        self.idel_y = idel_y * 0.5 ** np.arange(L)
        self.idel_z = idel_z * 0.5 ** np.arange(L)
        self.scalar_lambda = _is_scalar(lam)
        self.spatial = not (_is_scalar(D_xx) and _is_scalar(D_yy) and _is_scalar(D_zz))
        sqx, sqy, sqz = self.idel_x ** 2, self.idel_y ** 2, self.idel_z ** 2

        lam_l = None
        if not self.scalar_lambda:
            lam_l = [np.asarray(lam, dtype=np.float64)]
            for l in range(1, L):
                a = np.zeros(self.shapes[l])
                a[1:-1, 1:-1, 1:-1] = lam_l[l - 1][1::2, 1::2, 1::2]
                lam_l.append(a)
        self.lam_levels = lam_l

        if self.spatial:
            Dx = [np.array(D_xx, dtype=np.float64, copy=True)]
            Dy = [np.array(D_yy, dtype=np.float64, copy=True)]
            Dz = [np.array(D_zz, dtype=np.float64, copy=True)]
            for l in range(1, L):
                nx_, ny_, nz_ = (np.zeros(self.shapes[l]) for _ in range(3))
                nx_[1:-1, 1:-1, 1:-1] = Dx[l - 1][1::2, 1::2, 1::2]
                ny_[1:-1, 1:-1, 1:-1] = Dy[l - 1][1::2, 1::2, 1::2]
                nz_[1:-1, 1:-1, 1:-1] = Dz[l - 1][1::2, 1::2, 1::2]
                nx_[1:-1, 1:-1, :-1] = 0.5 * (nx_[1:-1, 1:-1, 1:] + nx_[1:-1, 1:-1, :-1])
                ny_[1:-1, :-1, 1:-1] = 0.5 * (ny_[1:-1, 1:, 1:-1] + ny_[1:-1, :-1, 1:-1])
                nz_[:-1, 1:-1, 1:-1] = 0.5 * (nz_[1:, 1:-1, 1:-1] + nz_[:-1, 1:-1, 1:-1])
                Dx.append(nx_)
                Dy.append(ny_)
                Dz.append(nz_)
            self.Dx, self.Dy, self.Dz = Dx, Dy, Dz
            self.lcc = [Dx[l][1:-1, 1:-1, 0:-2] * sqx[l] for l in range(L)]
            self.rcc = [Dx[l][1:-1, 1:-1, 1:-1] * sqx[l] for l in range(L)]
            self.clc = [Dy[l][1:-1, 0:-2, 1:-1] * sqy[l] for l in range(L)]
            self.crc = [Dy[l][1:-1, 1:-1, 1:-1] * sqy[l] for l in range(L)]
            self.ccl = [Dz[l][0:-2, 1:-1, 1:-1] * sqz[l] for l in range(L)]
            self.ccr = [Dz[l][1:-1, 1:-1, 1:-1] * sqz[l] for l in range(L)]
            self.ccc = [self.lcc[l] + self.rcc[l] + self.clc[l] + self.crc[l] + self.ccl[l] + self.ccr[l]
                        + (lam if self.scalar_lambda else lam_l[l][1:-1, 1:-1, 1:-1]) for l in range(L)]
        else:
            self.ax = float(D_xx) * sqx
            self.ay = float(D_yy) * sqy
            self.az = float(D_zz) * sqz
            add = 2 * (self.ax + self.ay + self.az)
            if self.scalar_lambda:
                self.ccc = add + lam
            else:
                self.ccc = [add[l] + lam_l[l][1:-1, 1:-1, 1:-1] for l in range(L)]

    def stencil(self, level):
        """Full-size (m_l+1)^3 coefficient arrays of one level."""
        s = self.shapes[level]
        shp = (s[0] - 2, s[1] - 2, s[2] - 2)
        if self.spatial:
            return dict(lcc=self.lcc[level], rcc=self.rcc[level], clc=self.clc[level],
                        crc=self.crc[level], ccl=self.ccl[level], ccr=self.ccr[level], ccc=self.ccc[level])
        ax, ay, az = self.ax[level], self.ay[level], self.az[level]
        return dict(lcc=np.full(shp, ax), rcc=np.full(shp, ax), clc=np.full(shp, ay), crc=np.full(shp, ay),
                    ccl=np.full(shp, az), ccr=np.full(shp, az),
                    ccc=np.broadcast_to(self.ccc[level], shp).copy())


class Oracle3D:
    """The reference's Solver_3D restated (solver_3d.py:239-706)."""

    def __init__(self, grid_x, grid_y, grid_z, fixed=False, epsilon=1e-12, gamma=1, fcycle=False,
                 skip_pre=False, nu1=1, nu2=1, max_iters_outer=INT32_MAX, max_iters_inner=INT32_MAX):
        self.fixed, self.epsilon, self.gamma, self.fcycle = fixed, epsilon, gamma, fcycle
        self.skip_pre, self.nu1, self.nu2 = skip_pre, nu1, nu2
        self.max_iters_outer, self.max_iters_inner = max_iters_outer, max_iters_inner
        self.levels, self.mxl, self.myl, self.mzl, self.shapes = level_layout(grid_x.mx, grid_y.mx, grid_z.mx)
        if not grid_x.is_linear or not grid_y.is_linear or not grid_z.is_linear:
            raise ValueError("Only linear grids are supported!")
        self.grids = (grid_x, grid_y, grid_z)
        self.h = None

    def setup(self, phi, rhs, lam, D_xx, D_yy, D_zz):
        arrs = [phi, rhs, lam, D_xx, D_yy, D_zz]
        if not all(np.asarray(a).dtype == np.float64 for a in arrs):
            raise ValueError("Incorrect configuration: dtype must be 'jnp.float64' for all arguments.")
        sl = _is_scalar(lam)
        spatial = not (_is_scalar(D_xx) and _is_scalar(D_yy) and _is_scalar(D_zz))
        s = np.shape
        if (not s(D_xx) == s(D_yy) == s(D_zz) or (sl and not s(phi) == s(rhs))
                or (not sl and not s(phi) == s(rhs) == s(lam))
                or (spatial and not s(phi) == s(rhs) == s(D_xx) == s(D_yy) == s(D_zz))
                or s(phi) != self.shapes[0]):
            raise ValueError(f"Shape mismatch: phi={s(phi)}, rhs={s(rhs)}, lam={s(lam)}, D_xx={s(D_xx)}, "
                             f"D_yy={s(D_yy)}, D_zz={s(D_zz)}.")
        gx, gy, gz = self.grids
        self.h = Hierarchy3D(gx.idel, gy.idel, gz.idel, gx.mx, gy.mx, gz.mx,
                             lam if sl else np.asarray(lam), D_xx, D_yy, D_zz)
        return self.h

    def rbgs(self, phi, rhs, level=0):
        """One sweep over the 8 sub-lattices in the reference order (solver_3d.py:679-706)."""
        h = self.h
        _zero_frame(phi)
        for (lx, ly, lz) in SUBLATTICES_3D:
            P = phi
            t = (slice(lz + 1, -1, 2), slice(ly + 1, -1, 2), slice(lx + 1, -1, 2))
            U = P[lz + 2::2, ly + 1:-1:2, lx + 1:-1:2]
            D = P[lz:-2:2, ly + 1:-1:2, lx + 1:-1:2]
            N = P[lz + 1:-1:2, ly + 2::2, lx + 1:-1:2]
            S = P[lz + 1:-1:2, ly:-2:2, lx + 1:-1:2]
            E = P[lz + 1:-1:2, ly + 1:-1:2, lx + 2::2]
            W = P[lz + 1:-1:2, ly + 1:-1:2, lx:-2:2]
            r = rhs[t]
            c = (slice(lz, None, 2), slice(ly, None, 2), slice(lx, None, 2))
            if h.spatial:
                new = (h.ccr[level][c] * U + h.ccl[level][c] * D + h.crc[level][c] * N + h.clc[level][c] * S
                       + h.rcc[level][c] * E + h.lcc[level][c] * W - r) / h.ccc[level][c]
            else:
                ax, ay, az = h.ax[level], h.ay[level], h.az[level]
                new = (az * U + az * D + ay * N + ay * S + ax * E + ax * W - r) / (
                    h.ccc[level] if h.scalar_lambda else h.ccc[level][c])
            phi[t] = new
            _zero_frame(phi)
        return phi

    def defect_field(self, phi, rhs, level):
        h = self.h
        d = np.zeros(rhs.shape)
        C = phi[1:-1, 1:-1, 1:-1]
        W, E = phi[1:-1, 1:-1, :-2], phi[1:-1, 1:-1, 2:]
        S, N = phi[1:-1, :-2, 1:-1], phi[1:-1, 2:, 1:-1]
        D, U = phi[:-2, 1:-1, 1:-1], phi[2:, 1:-1, 1:-1]
        r = rhs[1:-1, 1:-1, 1:-1]
        if h.spatial:
            d[1:-1, 1:-1, 1:-1] = (h.ccc[level] * C - h.lcc[level] * W - h.rcc[level] * E - h.clc[level] * S
                                   - h.crc[level] * N - h.ccl[level] * D - h.ccr[level] * U + r)
        else:
            ax, ay, az = h.ax[level], h.ay[level], h.az[level]
            d[1:-1, 1:-1, 1:-1] = h.ccc[level] * C - ax * W - ax * E - ay * S - ay * N - az * D - az * U + r
        return _zero_frame(d)

    def defect(self, phi, rhs, level):
        """Defect + restriction from the 12 edge-diagonal red neighbours (solver_3d.py:622-652)."""
        d = self.defect_field(phi, rhs, level)
        rc = np.zeros(self.shapes[level + 1])
        rc[1:-1, 1:-1, 1:-1] = 0.03125 * (
            d[1:-1:2, 2::2, 2::2] + d[1:-1:2, 2::2, :-2:2] + d[1:-1:2, :-2:2, 2::2] + d[1:-1:2, :-2:2, :-2:2]
            + d[2::2, 1:-1:2, 2::2] + d[2::2, 1:-1:2, :-2:2] + d[:-2:2, 1:-1:2, 2::2] + d[:-2:2, 1:-1:2, :-2:2]
            + d[2::2, 2::2, 1:-1:2] + d[2::2, :-2:2, 1:-1:2] + d[:-2:2, 2::2, 1:-1:2] + d[:-2:2, :-2:2, 1:-1:2]
        ) + 0.125 * d[1:-1:2, 1:-1:2, 1:-1:2]
        return _zero_frame(rc)

    def prolongate(self, phi_c, level):
        """solver_3d.py:654-677."""
        c = np.zeros(self.shapes[level])
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

    def cycle(self, phi, rhs, fcycle=False, level=0, skip_pre=False):
        """solver_3d.py:588-620, in place on ``phi``."""
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

    def solve(self, phi, rhs, lam, D_xx, D_yy, D_zz, callback=None):
        """solver_3d.py:431-486. Returns (phi, count)."""
        self.setup(phi, rhs, lam, D_xx, D_yy, D_zz)
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

    def rel_residual(self, phi, rhs):
        """||rhs - L_h phi||_2 / ||rhs||_2 over interior indices 2..m (FP64)."""
        d = self.defect_field(phi, rhs, 0)
        num = np.sqrt(np.sum(d[2:-2, 2:-2, 2:-2] ** 2))
        den = np.sqrt(np.sum(np.asarray(rhs)[2:-2, 2:-2, 2:-2] ** 2))
        return num / den


def solve_3d(grid_x, grid_y, grid_z, phi, rhs, lam, D_xx, D_yy, D_zz, *, fixed=False, epsilon=1e-12,
             gamma=1, fcycle=False, skip_pre=False, nu1=1, nu2=1, max_iters_outer=INT32_MAX,
             max_iters_inner=INT32_MAX):
    """Oracle counterpart of ``solve_3d`` (solver_3d.py:196-237)."""
    o = Oracle3D(grid_x, grid_y, grid_z, fixed=fixed, epsilon=epsilon, gamma=gamma, fcycle=fcycle,
                 skip_pre=skip_pre, nu1=nu1, nu2=nu2, max_iters_outer=max_iters_outer,
                 max_iters_inner=max_iters_inner)
    return o.solve(phi, rhs, lam, D_xx, D_yy, D_zz)
