"""The oracle pinned to the reference's own known answers (CPU only).

* every KAT of tests/test_solver_2d.py and tests/test_solver_3d.py: exact dynamic
  iteration count and RMSE within the reference's tolerance (approx rel 1e-9, abs 2e-15);
* the benchmark golden dictionaries (examples/benchmark.py:26-532) up to 128^2, except
  ``reference_wskip`` (95 of its 96 entries equal ``reference_vskip``'s), the entry
  (reference_v, 4, 64) whose RMSE contradicts the reference's own test4_64, and
  (reference_fskip, 9, 64), a D_xy problem one cycle off at the 1e-12 threshold;
* the C restatement bit-identical to the NumPy restatement.
"""
import numpy as np
import pytest

import problems as P
from oracle import c_oracle, mg2d, mg3d
from oracle.grid import OracleGrid1D as G

KNOWN_BAD = {("reference_v", 4, 64), ("reference_fskip", 9, 64)}
MODES = {"reference_v": {}, "reference_vskip": {"skip_pre": True}, "reference_f": {"fcycle": True},
         "reference_fskip": {"fcycle": True, "skip_pre": True}, "reference_w": {"gamma": 2}}


def _args2d(pid, mx, my):
    gx, gy, shape, pe, rhs, lam, D = P.make_2d(pid, mx, my, G)
    if np.ndim(lam) > 0:
        lam = np.broadcast_to(lam, shape).copy()
    D = [np.broadcast_to(a, shape).copy() if np.ndim(a) > 0 else a for a in D]
    return gx, gy, shape, pe, rhs, lam, D


def test_kat_2d_tests(goldens):
    for r in goldens["tests_2d"]:
        gx, gy, shape, pe, rhs, lam, D = _args2d(r["problem"], *r["res"])
        if len(D) == 3:  # D_xy problems: NumPy oracle (the C restatement has no 9-point stencil)
            if r["iterations"] > 300:
                continue  # the 300-800 cycle D_xy cases run in the slow suite
            phi, c = mg2d.solve_2d(gx, gy, np.zeros(shape), rhs, lam, D[0], D[1], D_xy=D[2])
        else:
            phi, c, _ = c_oracle.solve((gx, gy), np.zeros(shape), rhs, lam, D)
        assert c == r["iterations"], r["test"]
        assert P.rmse(pe, phi) == pytest.approx(r["rmse"], abs=2e-15, rel=1e-9), r["test"]


@pytest.mark.slow
def test_kat_2d_dxy_long(goldens):
    for r in goldens["tests_2d"]:
        gx, gy, shape, pe, rhs, lam, D = _args2d(r["problem"], *r["res"])
        if len(D) != 3 or r["iterations"] <= 300:
            continue
        phi, c = mg2d.solve_2d(gx, gy, np.zeros(shape), rhs, lam, D[0], D[1], D_xy=D[2])
        assert c == r["iterations"], r["test"]
        assert P.rmse(pe, phi) == pytest.approx(r["rmse"], abs=2e-15, rel=1e-9), r["test"]


def test_kat_3d_tests(goldens):
    for r in goldens["tests_3d"]:
        gx, gy, gz, shape, pe, rhs, lam, D = P.make_3d(r["problem"], *r["res"], G)
        phi, c, _ = c_oracle.solve((gx, gy, gz), np.zeros(shape), rhs, lam, D)
        assert c == r["iterations"], r["test"]
        assert P.rmse(pe, phi) == pytest.approx(r["rmse"], abs=2e-15, rel=1e-9), r["test"]


def test_kat_3d_numpy_oracle(goldens):
    for r in goldens["tests_3d"]:
        if max(r["res"]) > 32:
            continue
        gx, gy, gz, shape, pe, rhs, lam, D = P.make_3d(r["problem"], *r["res"], G)
        phi, c = mg3d.solve_3d(gx, gy, gz, np.zeros(shape), rhs, lam, *D)
        assert c == r["iterations"], r["test"]
        assert P.rmse(pe, phi) == pytest.approx(r["rmse"], abs=2e-15, rel=1e-9), r["test"]


@pytest.mark.parametrize("mode", sorted(MODES))
def test_benchmark_dictionaries(goldens, mode):
    n = 0
    for r in goldens["benchmark_2d"][mode]:
        if r["res"] > 128 or (mode, r["problem"], r["res"]) in KNOWN_BAD:
            continue
        gx, gy, shape, pe, rhs, lam, D = _args2d(r["problem"], r["res"], r["res"])
        if len(D) == 3:
            if r["iterations"] > 250:
                continue
            phi, c = mg2d.solve_2d(gx, gy, np.zeros(shape), rhs, lam, D[0], D[1], D_xy=D[2], **MODES[mode])
        else:
            phi, c, _ = c_oracle.solve((gx, gy), np.zeros(shape), rhs, lam, D, **MODES[mode])
        assert c == r["iterations"], (mode, r["problem"], r["res"])
        if r["rmse"] is not None:
            assert P.rmse(pe, phi) == pytest.approx(r["rmse"], rel=1e-9), (mode, r["problem"], r["res"])
        n += 1
    assert n >= 20


def test_wskip_dictionary_is_a_copy_of_vskip(goldens):
    v = {(r["problem"], r["res"]): (r["iterations"], r["rmse"]) for r in goldens["benchmark_2d"]["reference_vskip"]}
    w = {(r["problem"], r["res"]): (r["iterations"], r["rmse"]) for r in goldens["benchmark_2d"]["reference_wskip"]}
    diff = sorted(k for k in v if v[k] != w.get(k))
    assert diff == [(9, 16384)]  # 95 of 96 entries are identical


def test_known_bad_entry_contradicts_reference_test(goldens):
    t = next(r for r in goldens["tests_2d"] if r["test"] == "test4_64")
    b = next(r for r in goldens["benchmark_2d"]["reference_v"] if (r["problem"], r["res"]) == (4, 64))
    assert t["iterations"] == b["iterations"] and abs(t["rmse"] - b["rmse"]) / t["rmse"] > 0.5


@pytest.mark.parametrize("kw", [{}, {"gamma": 2}, {"fcycle": True}, {"skip_pre": True}, {"nu1": 2, "nu2": 0},
                                {"nu1": 0, "nu2": 1}])
def test_c_oracle_bit_identical_2d(kw):
    for pid in (1, 3, 4, 5):
        gx, gy, shape, pe, rhs, lam, D = _args2d(pid, 32, 64)
        a, _ = mg2d.solve_2d(gx, gy, np.zeros(shape), rhs, lam, D[0], D[1], fixed=True, max_iters_outer=5, **kw)
        b, _, _ = c_oracle.solve((gx, gy), np.zeros(shape), rhs, lam, D[:2], fixed=True, max_iters_outer=5, **kw)
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("kw", [{}, {"gamma": 2}, {"fcycle": True}, {"nu1": 1, "nu2": 0}])
def test_c_oracle_bit_identical_3d(kw):
    for pid in (1, 2, 3):
        gx, gy, gz, shape, pe, rhs, lam, D = P.make_3d(pid, 16, 8, 16, G)
        a, _ = mg3d.solve_3d(gx, gy, gz, np.zeros(shape), rhs, lam, *D, fixed=True, max_iters_outer=4, **kw)
        b, _, _ = c_oracle.solve((gx, gy, gz), np.zeros(shape), rhs, lam, D, fixed=True, max_iters_outer=4, **kw)
        np.testing.assert_array_equal(a, b)
    from jsolver_gb300 import workloads as W
    p = W.random_3d(16, seed=4)
    g = G(16)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
    a, _ = mg3d.solve_3d(g, g, g, *args, fixed=True, max_iters_outer=3, **kw)
    b, _, _ = c_oracle.solve((g, g, g), args[0], args[1], args[2], args[3:], fixed=True, max_iters_outer=3, **kw)
    np.testing.assert_array_equal(a, b)


def test_c_oracle_dynamic_and_residual_stop():
    from jsolver_gb300 import workloads as W
    p = W.random_2d(64, seed=2)
    g = G(64)
    args = (p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    a, ca = mg2d.solve_2d(g, g, *args)
    b, cb, _ = c_oracle.solve((g, g), args[0], args[1], args[2], args[3:])
    assert ca == cb
    np.testing.assert_array_equal(a, b)
    b, cb, rr = c_oracle.solve((g, g), args[0], args[1], args[2], args[3:], stop="residual", rtol=1e-10)
    o = mg2d.Oracle2D(g, g)
    o.setup(*args)
    assert rr <= 1e-10 and o.rel_residual(b, p["rhs"]) == pytest.approx(rr, rel=1e-6)
    # one cycle fewer is not yet converged
    c2, _, rr2 = c_oracle.solve((g, g), args[0], args[1], args[2], args[3:], fixed=True, max_iters_outer=cb - 1)
    assert rr2 > 1e-10
