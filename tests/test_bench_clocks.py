"""bench.py's clock record (CPU): the NVML sampler's summary from fake samples, and the fallback
when neither NVML nor nvidia-smi is present."""
from __future__ import annotations

import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402


class FakeNvml:
    max_mhz = 2070.0


def test_nvml_summary_reports_median_and_reasons():
    c = bench.ClockSampler(0)
    c.nvml = FakeNvml()
    # SM clocks with sw_power_cap (0x4) once and hw_slowdown (0x8) once.
    c.samples = [(2070.0, 0), (2055.0, 0x4), (2070.0, 0), (1980.0, 0x8 | 0x1)]
    s = c.summary()
    assert s["sm_mhz"] == 2062.5 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 4
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"] and s["source"] == "nvml"


def test_summary_without_any_sampler_is_empty():
    c = bench.ClockSampler(0)
    s = c.summary()
    assert s["sm_mhz"] is None and s["samples"] == 0 and s["reasons"] == []
