"""Which initial-guess errors cost cycles: the reference's iteration on a 2D random-
coefficient problem (C oracle, CPU), residual stop 1e-10.

This is the measurement behind the learned guess's result. Starting from the exact
discrete solution with a small error added, the plain multigrid needs MORE cycles than
from zero when the error is generic (white noise of 0.4 % of the solution's RMS, or a
relative 4e-3 per point, the size of BF16 rounding), because such errors reach the slow
modes of this smoother and coarse-grid correction (injected coarse operators on rough
coefficients), which the smooth manufactured solution barely excites. An error
proportional to the solution itself is removed at the solution's own rate and saves
cycles. A BF16 network's guess errs the first way.
"""
import numpy as np
import pytest

from jsolver_gb300 import workloads as W
from oracle import c_oracle
from oracle.grid import OracleGrid1D


def _cycles(m, p, g, phi0):
    _, cnt, rr = c_oracle.solve((g, g), phi0, p["rhs"], p["lam"], (p["D_xx"], p["D_yy"]), stop="residual", rtol=1e-10)
    assert rr <= 1e-10
    return cnt


def _frame0(a):
    a = a.copy()
    a[:2] = 0
    a[-2:] = 0
    a[:, :2] = 0
    a[:, -2:] = 0
    return a


@pytest.mark.parametrize("seed", [2, 3])
def test_generic_small_errors_cost_cycles(seed):
    m = 256
    p = W.random_2d(m, seed=seed)
    g = OracleGrid1D(m)
    ex = p["phi_exact"]
    rng = np.random.default_rng(seed)
    rms = np.sqrt(np.mean(ex ** 2))
    zero = _cycles(m, p, g, np.zeros_like(ex))
    white = _cycles(m, p, g, _frame0(ex + 4e-3 * rms * rng.standard_normal(ex.shape)))
    bf16 = _cycles(m, p, g, _frame0(ex * (1 + 4e-3 * rng.standard_normal(ex.shape))))
    scaled = _cycles(m, p, g, 0.84 * ex)
    assert white > zero and bf16 > zero, (zero, white, bf16)
    assert scaled < zero, (zero, scaled)
