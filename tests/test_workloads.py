"""Synthetic workloads: the manufactured rhs makes phi* the exact discrete solution."""
import numpy as np

from jsolver_gb300 import workloads as W
from oracle import mg2d, mg3d
from oracle.grid import OracleGrid1D as G


def test_random_2d_exact_discrete_solution():
    p = W.random_2d(64, seed=1)
    o = mg2d.Oracle2D(G(64), G(64))
    o.setup(p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"])
    d = o.defect_field(p["phi_exact"], p["rhs"], 0)
    assert np.abs(d).max() <= 1e-12 * np.abs(p["rhs"]).max() * 64
    assert p["D_xx"].shape == (67, 67) and p["lam"].min() >= 0 and p["lam"].max() <= 10


def test_random_2d_is_seeded():
    a, b, c = W.random_2d(32, seed=3), W.random_2d(32, seed=3), W.random_2d(32, seed=4)
    np.testing.assert_array_equal(a["D_xx"], b["D_xx"])
    assert not np.array_equal(a["D_xx"], c["D_xx"])


def test_grf_statistics():
    g = W.grf((515, 515), 1 / 512, 0.05, 1.0, np.random.default_rng(0))
    assert abs(g.mean()) < 1e-12 and abs(g.std() - 1.0) < 1e-12
    # correlation at one correlation length is well above zero, far away it is small
    c1 = np.mean(g[:, :-26] * g[:, 26:])
    c5 = np.mean(g[:, :-128] * g[:, 128:])
    assert c1 > 0.3 and abs(c5) < 0.2


def test_random_3d_shapes():
    p = W.random_3d(16, seed=0)
    assert p["rhs"].shape == (19, 19, 19)
    assert p["lam"].min() == 0.0 and abs(p["lam"].max() - 50.0) < 1e-12
    assert np.all(p["rhs"][:2] == 0) and np.all(p["rhs"][:, :, -2:] == 0)
    o = mg3d.Oracle3D(G(16), G(16), G(16))
    o.setup(p["phi0"], p["rhs"], p["lam"], p["D_xx"], p["D_yy"], p["D_zz"])
    assert o.rel_residual(p["phi0"], p["rhs"]) == 1.0
