"""grid_1D and do_BCs known answers (reference tests/test_grid_1d.py:9-52,
tests/test_boundary_handler_2d.py:60-119), for the product classes (host side)."""
import numpy as np
import pytest

from jsolver_gb300.boundary_handler_2d import do_BCs as bc2
from jsolver_gb300.boundary_handler_3d import do_BCs as bc3
from jsolver_gb300.grid_1d import grid_1D
from oracle import mg2d, mg3d


@pytest.fixture
def grid():
    return grid_1D(mx=128, xb=0., xe=1., rim=1, grid_type=0, centered=True)


def test_init_and_dependent_values(grid):
    assert (grid.mx, grid.nx, grid.centered, grid.rim, grid.xb, grid.xe, grid.grid_type) == (128, 129, True, 1, 0.0, 1.0, 0)
    assert grid.length == 1.0
    assert grid.del_ == pytest.approx(0.0078125)
    assert grid.idel == pytest.approx(128.0)


def test_array_values(grid):
    assert grid.centers[0] == pytest.approx(-0.0078125)
    assert grid.centers[-1] == pytest.approx(1.0078125)
    assert grid.edges[0] == pytest.approx(-0.01171875)
    assert grid.edges[-1] == pytest.approx(1.01171875)
    assert grid.widths[0] == pytest.approx(0.0078125)
    assert grid.widths[-1] == pytest.approx(0.0078125)
    assert grid.centers.size == grid.widths.size == grid.edges.size - 1 == 131
    assert grid.centers[1] == 0.0 and grid.centers[129] == 1.0


def test_hash_eq(grid):
    assert grid == grid_1D(128) and hash(grid) == hash(grid_1D(128))
    assert grid != grid_1D(64) and grid != grid_1D(128, xe=2.0)


def test_sinusoidal():
    g = grid_1D(mx=128, xb=0., xe=1., rim=1, grid_type=1)
    assert g.centers[0] == pytest.approx(-0.00428662)
    assert g.centers[-1] == pytest.approx(1.0121)
    assert g.edges[0] == pytest.approx(-0.00857324)
    assert g.edges[-1] == pytest.approx(1.01639, rel=1e-5)
    assert g.widths[0] == pytest.approx(0.00857324)
    assert not g.is_linear


def test_unknown_grid_type():
    with pytest.raises(ValueError, match="No such grid grid_type: 42"):
        grid_1D(mx=128, grid_type=42)


def test_bcs_2d_default_and_values():
    dim = 131
    new = bc2(np.ones((dim, dim)))
    for idx in (0, 1, -1, -2):
        assert np.all(new[idx] == 0) and np.all(new[:, idx] == 0)
    assert np.all(new[2:-2, 2:-2] == 1)
    twos = np.ones(dim) * 2
    new = bc2(np.ones((dim, dim)), vals_xb=twos, vals_xe=twos, vals_yb=twos, vals_ye=twos)
    for idx in (0, 1, -1, -2):
        assert np.all(new[idx] == twos) and np.all(new[:, idx] == twos)


def test_bcs_2d_directions():
    dim = 131
    pad = np.pad(np.ones(dim - 4), (2, 2))
    new = bc2(np.ones((dim, dim)), direction=0)
    for idx in (0, 1, -1, -2):
        assert np.all(new[idx] == pad) and np.all(new[:, idx] == 0)
    new = bc2(np.ones((dim, dim)), direction=1)
    for idx in (0, 1, -1, -2):
        assert np.all(new[idx] == 0) and np.all(new[:, idx] == pad)


def test_bcs_match_oracle():
    a = np.random.default_rng(0).standard_normal((19, 23))
    np.testing.assert_array_equal(bc2(a), mg2d.do_bcs(a))
    b = np.random.default_rng(1).standard_normal((7, 11, 13))
    np.testing.assert_array_equal(bc3(b), mg3d.do_bcs(b))
    v = np.random.default_rng(2).standard_normal((7, 13))
    np.testing.assert_array_equal(bc3(b, vals_yb=v, vals_ye=v, direction=1),
                                  mg3d.do_bcs(b, vals_yb=v, vals_ye=v, direction=1))
