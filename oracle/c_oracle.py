"""ctypes front end of the C oracle (test infrastructure; see jmg_oracle.c)."""
import ctypes
import os

import numpy as np

from . import build_c

_lib = None
_P = ctypes.c_void_p


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build_c.build())
        lib.jmgo_solve.restype = ctypes.c_int64
        lib.jmgo_solve.argtypes = [ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_double, _P, _P, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.c_double, _P, _P, ctypes.c_int]
        lib.jmgo_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


def solve(grids, phi, rhs, lam, D, fixed=False, epsilon=1e-12, gamma=1, fcycle=False, skip_pre=False, nu1=1,
          nu2=1, max_iters_outer=2147483647, stop="distance", rtol=1e-10, nthreads=0):
    """Returns (phi, count, final relative residual). Same conventions as solve_2d/3d."""
    lib = load()
    dim = len(grids)
    m = np.array([g.mx for g in grids], dtype=np.int32)
    idel = np.array([g.idel for g in grids], dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    rhs = np.ascontiguousarray(rhs, dtype=np.float64)
    lam_arr = None if np.ndim(lam) == 0 else np.ascontiguousarray(lam, dtype=np.float64)
    lam_s = float(lam) if lam_arr is None else 0.0
    scalar = all(np.ndim(d) == 0 for d in D)
    Darr = [None if scalar else np.ascontiguousarray(d, dtype=np.float64) for d in D]
    Dptr = (ctypes.c_void_p * 3)(*[(_p(a).value if a is not None else None) for a in Darr] + [None] * (3 - dim))
    Ds = np.array([float(d) if scalar else 0.0 for d in D] + [0.0] * (3 - dim))
    out = np.empty_like(phi)
    rr = np.zeros(1)
    cnt = lib.jmgo_solve(dim, _p(m), _p(idel), _p(phi), _p(rhs), _p(lam_arr), lam_s, Dptr, _p(Ds), int(fixed),
                         float(epsilon), int(gamma), int(fcycle), int(skip_pre), int(nu1), int(nu2),
                         int(max_iters_outer), 1 if stop == "residual" else 0, float(rtol), _p(out), _p(rr),
                         int(nthreads))
    if cnt < 0:
        raise ValueError("bad arguments to the C oracle")
    return out, int(cnt), float(rr[0])


def max_threads():
    return load().jmgo_max_threads()
