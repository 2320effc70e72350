"""Host logic of bench.py that needs no GPU: the timed form's smoothing counts and the
clock sampler (NVML through a fake library, and the nvidia-smi CSV fallback)."""
import ctypes
import os
import sys
import types

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _args(**kw):
    a = dict(outer="fcg", form="mixed", nu1=None, nu2=None)
    a.update(kw)
    return types.SimpleNamespace(**a)


def test_form_nu_defaults_and_overrides():
    assert bench.form_nu(_args(), 2) == (1, 5)
    assert bench.form_nu(_args(), 3) == (1, 3)
    assert bench.form_nu(_args(form="learned-mixed"), 2) == (1, 5)
    # the reference's iteration and the plain forms keep (1, 1)
    assert bench.form_nu(_args(outer="richardson"), 2) == (1, 1)
    assert bench.form_nu(_args(form="fp64"), 3) == (1, 1)
    assert bench.form_nu(_args(nu1=2, nu2=4), 2) == (2, 4)


class _FakeNvml:
    """The NVML calls the sampler makes; every output goes through the byref argument."""

    def __init__(self, clocks, reasons, uuid_ok=True):
        self.clocks = list(clocks)
        self.reasons = reasons
        self.uuid_ok = uuid_ok
        self.calls = []
        self.shut = False

    def nvmlInit_v2(self):
        return 0

    def nvmlShutdown(self):
        self.shut = True
        return 0

    def nvmlDeviceGetHandleByUUID(self, uuid, h):
        self.calls.append(("uuid", uuid))
        if not self.uuid_ok:
            return 13
        h._obj.value = 1234
        return 0

    def nvmlDeviceGetHandleByIndex_v2(self, idx, h):
        self.calls.append(("index", idx.value))
        h._obj.value = 1234
        return 0

    def nvmlDeviceGetMaxClockInfo(self, h, kind, out):
        out._obj.value = 2070
        return 0

    def nvmlDeviceGetClockInfo(self, h, kind, out):
        assert kind == bench.Clocks.NVML_CLOCK_SM
        out._obj.value = self.clocks.pop(0) if len(self.clocks) > 1 else self.clocks[0]
        return 0

    def nvmlDeviceGetCurrentClocksEventReasons(self, h, out):
        out._obj.value = self.reasons
        return 0


def test_clocks_nvml_reasons_and_median(monkeypatch):
    fake = _FakeNvml([2070, 1980, 2070], 0x4 | 0x40 | 0x1)  # power cap, hw thermal, idle
    monkeypatch.setattr(ctypes, "CDLL", lambda name: fake)
    monkeypatch.setattr(bench.Clocks, "POLL_S", 0.001)
    with bench.Clocks(0, "70e5bcd2-c010-186b-0902-e0ead956353e") as c:
        pass
    s = c.summary()
    assert s["source"] == "nvml" and s["sm_max_mhz"] == 2070.0
    assert s["samples"] >= 1 and s["sm_mhz"] in (1980.0, 2070.0)
    # the idle bit is not a throttle reason; the others keep their nvidia-smi names
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert fake.calls[0] == ("uuid", b"GPU-70e5bcd2-c010-186b-0902-e0ead956353e")
    assert fake.shut


def test_clocks_nvml_falls_back_to_the_index(monkeypatch):
    fake = _FakeNvml([2070], 0, uuid_ok=False)
    monkeypatch.setattr(ctypes, "CDLL", lambda name: fake)
    with bench.Clocks(3, "00000000-0000-0000-0000-000000000000") as c:
        pass
    assert ("index", 3) in fake.calls
    s = c.summary()
    assert s["reasons"] == [] and s["sm_mhz"] == 2070.0


def test_clocks_nvidia_smi_csv(monkeypatch):
    def no_nvml(name):
        raise OSError("no NVML here")

    class _Proc:
        def __init__(self, *a, **k):
            pass

        def terminate(self):
            pass

        def communicate(self, timeout=None):
            rows = ["0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
                    "0, 1800, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
                    "0, 2070, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
                    "garbage line"]
            return "\n".join(rows), ""

    monkeypatch.setattr(ctypes, "CDLL", no_nvml)
    monkeypatch.setattr(bench.subprocess, "Popen", _Proc)
    with bench.Clocks(0, None) as c:
        pass
    s = c.summary()
    assert s["source"] == "nvidia-smi"
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["min_sm_mhz"] == 1800.0
    assert s["reasons"] == ["sw_power_cap"]


@pytest.mark.parametrize("raw,want", [("70e5bcd2-c010-186b-0902-e0ead956353e", "70e5bcd2-c010-186b-0902-e0ead956353e"),
                                      ("GPU-70e5bcd2-c010", "70e5bcd2-c010"),
                                      ("not a uuid", None)])
def test_gpu_uuid_normalises(monkeypatch, raw, want):
    import torch
    monkeypatch.setattr(torch.cuda, "get_device_properties", lambda dev: types.SimpleNamespace(uuid=raw))
    assert bench.gpu_uuid(0) == want
