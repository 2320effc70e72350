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


def test_config_extensions_are_validated_without_gpu():
    """outer='fcg' needs the residual stop or a fixed count; off_diag is 2D only; the
    workspace grows by the FCG vectors and the D_xy diagonals (plan layout is host-only)."""
    import pytest
    g2 = _engine.make_grid((grid_1D(64), grid_1D(64)))
    g3 = _engine.make_grid((grid_1D(16),) * 3)
    with pytest.raises(ValueError, match="fcg"):
        _lib.Plan(g2, _engine.make_config(outer="fcg"))
    with pytest.raises(ValueError, match="outer"):
        _engine.make_config(outer="gmres")
    with pytest.raises(ValueError, match="2D"):
        _lib.Plan(g3, _engine.make_config(off_diag=True))
    base = _lib.Plan(g2, _engine.make_config(stop="residual")).workspace_bytes
    fcg = _lib.Plan(g2, _engine.make_config(stop="residual", outer="fcg")).workspace_bytes
    fixed_fcg = _lib.Plan(g2, _engine.make_config(fixed=True, outer="fcg")).workspace_bytes
    dxy = _lib.Plan(g2, _engine.make_config(off_diag=True)).workspace_bytes
    n0 = 67 * 80 * 8  # level-0 FP64 array (pitch 80)
    assert fcg >= base + 4 * n0 and fixed_fcg == fcg
    assert dxy >= base + 4 * n0  # four diagonal couplings per level


def test_launch_counts_follow_the_form(monkeypatch):
    monkeypatch.setenv("JMG_FUSED", "0")  # the same sweeps in both forms
    monkeypatch.setenv("JMG_FUSEDOPS", "0")  # and the same operators
    lib = _lib.load()
    g = _engine.make_grid((grid_1D(1024), grid_1D(1024)))
    counts = {}
    for name, cfg in (("plain", _engine.make_config(stop="residual")),
                      ("fcg", _engine.make_config(stop="residual", precision="mixed", outer="fcg"))):
        p = _lib.Plan(g, cfg)
        a, b = ctypes.c_int64(), ctypes.c_int64()
        assert lib.jmg_plan_launch_counts(p.handle, ctypes.byref(a), ctypes.byref(b)) == 0
        counts[name] = b.value
    # an FCG step adds its four vector kernels to the cycle and the stopping test
    assert counts["fcg"] >= counts["plain"] + 3


def test_fused_operator_pairs_cut_launches(monkeypatch):
    """2D grid-wide levels run smooth + restrict and prolong + smooth as two fused
    launches per visit instead of six (two colour passes per sweep, restriction,
    prolongation): every FP32 level, FP64 levels up to 2^19 padded points."""
    lib = _lib.load()
    g = _engine.make_grid((grid_1D(1024), grid_1D(1024)))
    monkeypatch.setenv("JMG_FUSED2D", "0")  # colour passes wherever a level sweeps on its own

    def per_cycle(env, **kw):
        monkeypatch.delenv("JMG_FUSEDOPS", raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        p = _lib.Plan(g, _engine.make_config(**kw))
        a, b = ctypes.c_int64(), ctypes.c_int64()
        assert lib.jmg_plan_launch_counts(p.handle, ctypes.byref(a), ctypes.byref(b)) == 0
        return b.value

    # V(1,1) over 11 levels: levels 0 .. 4 grid-wide (6 launches each unfused, 2 fused)
    fp32_off = per_cycle({"JMG_FUSEDOPS": "0"}, stop="residual", precision="mixed", outer="fcg", inner_cycles=1)
    fp32_on = per_cycle({}, stop="residual", precision="mixed", outer="fcg", inner_cycles=1)
    assert fp32_off - fp32_on == 5 * 4
    fp64_off = per_cycle({"JMG_FUSEDOPS": "0"})
    fp64_on = per_cycle({})
    assert fp64_off - fp64_on == 4 * 4  # level 0 (1027^2 points) is not fused in FP64


def test_sweep_launches_per_level(monkeypatch):
    """One-pass sweeps: 3D levels whose one-pass grid fills half a wave (256^3 and finer),
    the 2D grid-wide levels (more padded points than the coarse block takes; off with
    JMG_FUSED2D=0), FP32 by default, FP64 with JMG_FUSED64=1, none with JMG_FUSED=0 or with
    D_xy; each has a second phi buffer. JMG_FUSED_POINTS selects levels by size instead."""
    lib = _lib.load()
    for k in ("JMG_FUSED", "JMG_FUSED64", "JMG_FUSED_POINTS", "JMG_FUSED2D"):
        monkeypatch.delenv(k, raising=False)
    g3 = _engine.make_grid((grid_1D(256),) * 3)
    mixed = _engine.make_config(precision="mixed")
    p = _lib.Plan(g3, mixed)
    assert lib.jmg_plan_sweep_launches(p.handle, 0, 1) == 1   # 259^3 padded: one pass
    assert lib.jmg_plan_sweep_launches(p.handle, 1, 1) == 2   # 131^3: colour passes
    assert lib.jmg_plan_sweep_launches(p.handle, 0, 0) == 2   # FP64 levels: colour passes
    assert lib.jmg_plan_sweep_launches(p.handle, 99, 1) == 0
    monkeypatch.setenv("JMG_FUSED", "0")
    off = _lib.Plan(g3, mixed)
    assert lib.jmg_plan_sweep_launches(off.handle, 0, 1) == 2
    assert off.workspace_bytes < p.workspace_bytes  # no second FP32 buffer
    monkeypatch.delenv("JMG_FUSED")
    monkeypatch.setenv("JMG_FUSED64", "1")
    assert lib.jmg_plan_sweep_launches(_lib.Plan(g3, mixed).handle, 0, 0) == 1
    monkeypatch.setenv("JMG_FUSED_POINTS", "100000")
    small = _lib.Plan(_engine.make_grid((grid_1D(64),) * 3), mixed)
    assert [lib.jmg_plan_sweep_launches(small.handle, lv, 1) for lv in range(3)] == [1, 2, 2]
    monkeypatch.delenv("JMG_FUSED_POINTS")
    g2 = _engine.make_grid((grid_1D(1024),) * 2)
    p2 = _lib.Plan(g2, mixed)
    # 2D: the grid-wide levels 1024^2 .. 64^2 sweep in one pass, the coarse block's levels
    # (35^2 = 1225 padded points and fewer) in colour passes
    assert [lib.jmg_plan_sweep_launches(p2.handle, lv, 1) for lv in range(7)] == [1, 1, 1, 1, 1, 2, 2]
    monkeypatch.setenv("JMG_FUSED2D", "0")
    assert [lib.jmg_plan_sweep_launches(_lib.Plan(g2, mixed).handle, lv, 1) for lv in range(3)] == [2, 2, 2]
    assert lib.jmg_plan_sweep_launches(_lib.Plan(g2, _engine.make_config(off_diag=True)).handle, 0, 0) == 4
