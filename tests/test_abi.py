"""The C-ABI library loads and exports every function declared in include/jmg.h (no GPU needed)."""
import ctypes
import os
import re

from jsolver_gb300 import _engine, _lib
from jsolver_gb300.grid_1d import grid_1D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "jmg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(jmg_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    lib = _lib.load()
    names = declared()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib._SIGS, f"{n} has no ctypes signature"


def test_plan_is_host_only():
    p = _lib.Plan(_engine.make_grid((grid_1D(1024), grid_1D(1024))), _engine.make_config())
    assert p.levels == 11 and p.workspace_bytes > 6 * 1027 * 1027 * 8
    a, b = ctypes.c_int64(), ctypes.c_int64()
    assert _lib.load().jmg_plan_launch_counts(p.handle, ctypes.byref(a), ctypes.byref(b)) == 0
    assert a.value > 0 and b.value > 0


def test_workspace_and_argument_errors_without_gpu():
    lib = _lib.load()
    p = _lib.Plan(_engine.make_grid((grid_1D(16), grid_1D(16))), _engine.make_config())
    co = _lib.JmgCoeffs()
    rc = lib.jmg_solve(p.handle, None, None, ctypes.byref(co), None, None, None, 0, None)
    assert rc == _lib.JMG_ERR_WORKSPACE and b"workspace" in lib.jmg_last_error()
    cfg = _engine.make_config()
    g = _lib.JmgGrid()
    g.ndim = 4
    h = ctypes.c_void_p()
    assert lib.jmg_plan_create(ctypes.byref(h), ctypes.byref(g), ctypes.byref(cfg)) == _lib.JMG_ERR_VALUE


def test_too_small_grid_is_a_value_error():
    import pytest
    with pytest.raises(ValueError, match="too small"):
        _lib.Plan(_engine.make_grid((grid_1D(1), grid_1D(1))), _engine.make_config())
