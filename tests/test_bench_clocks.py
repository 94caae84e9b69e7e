"""The clock record of bench.py, parsed from nvidia-smi's CSV on the CPU.

A run is judged by the SM clocks and throttle reasons sampled during its
timed region, so the parser must report the median SM clock, the highest
maximum clock and every active reason (hw_slowdown, hw_thermal_slowdown,
sw_thermal_slowdown, sw_power_cap), skip lines it cannot read, and say so
when nothing was sampled.  The sampler itself needs a GPU; here its output
file is written by the test.
"""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

import bench  # noqa: E402


def _summary(tmp_path, text):
    s = bench.ClockSampler(0)
    s.path = str(tmp_path / "clocks.csv")
    Path(s.path).write_text(text)
    return s.summary()


def test_steady_clocks_and_power_cap(tmp_path):
    rows = [
        "0, 2070, 2070, 1180.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1390.2, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1201.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
    ]
    got = _summary(tmp_path, "\n".join(rows) + "\n")
    assert got["sm_mhz"] == 2070.0
    assert got["sm_max_mhz"] == 2070.0
    assert got["reasons"] == ["sw_power_cap"]
    assert got["samples"] == 3


def test_thermal_and_hardware_slowdowns_are_reported(tmp_path):
    rows = [
        "0, 1500, 2070, 1000.0, 0x0000000000000048, Active, Not Active, Not Active, Not Active",
        "0, 1410, 2070, 1000.0, 0x0000000000000020, Not Active, Active, Active, Not Active",
    ]
    got = _summary(tmp_path, "\n".join(rows) + "\n")
    assert got["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert got["sm_mhz"] == 1455.0


def test_unreadable_lines_are_skipped(tmp_path):
    rows = [
        "garbage",
        "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]",
        "0, 1980, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    got = _summary(tmp_path, "\n".join(rows) + "\n")
    assert got["sm_mhz"] == 1980.0          # the [N/A] row has no clock to count
    assert got["samples"] == 2              # both nine-field rows were read
    assert got["reasons"] == []


def test_no_samples(tmp_path):
    got = _summary(tmp_path, "")
    assert got["sm_mhz"] is None and got["reasons"] == ["no nvidia-smi samples"]
