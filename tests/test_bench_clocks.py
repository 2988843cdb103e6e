"""bench.py's clock record: the NVML sampler's summary (median SM clock, the
maximum, the union of the clocks-event reasons seen) and the fallback when
NVML is unavailable, checked on CPU against a fake NVML reader (no GPU
setting is read or changed)."""
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class _FakeNvml:
    def __init__(self, index):
        self.max_mhz = 2070.0
        self.k = 0
        self.seq = [(2070.0, []), (2055.0, ["sw_power_cap"]), (2070.0, []), (1995.0, ["hw_slowdown"])]

    def sample(self):
        v = self.seq[self.k % len(self.seq)]
        self.k += 1
        return v


def test_nvml_summary(monkeypatch):
    monkeypatch.setattr(bench, "NvmlClocks", _FakeNvml)
    with bench.ClockSampler(0) as c:
        time.sleep(0.03)
    s = c.summary()
    assert s["source"].startswith("nvml")
    assert s["samples"] >= 2
    assert s["sm_max_mhz"] == 2070.0
    assert 1995.0 <= s["sm_mhz"] <= 2070.0
    assert set(s["reasons"]) <= {"sw_power_cap", "hw_slowdown"}
    assert "sw_power_cap" in s["reasons"]     # the second sample (entry and exit always sample)


def test_nvml_unavailable_falls_back(monkeypatch):
    def broken(index):
        raise OSError("NVML unavailable")
    monkeypatch.setattr(bench, "NvmlClocks", broken)
    monkeypatch.setenv("PATH", "/nonexistent")      # no nvidia-smi either
    with bench.ClockSampler(0) as c:
        pass
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_reason_bits_match_nvml_header():
    # nvml.h: SwPowerCap 0x4, HwSlowdown 0x8, SwThermalSlowdown 0x20,
    # HwThermalSlowdown 0x40, HwPowerBrakeSlowdown 0x80
    r = bench.NvmlClocks.REASONS
    assert r[0x4] == "sw_power_cap" and r[0x8] == "hw_slowdown" and r[0x20] == "sw_thermal_slowdown"
    assert r[0x40] == "hw_thermal_slowdown" and r[0x80] == "hw_power_brake_slowdown"
