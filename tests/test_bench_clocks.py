"""The bench's clock sampler, against a stand-in for nvidia-smi that prints
samples with chosen timestamps: it keeps the samples stamped inside the timed
loop, falls back to all samples when none is, and reports the throttle
reasons of the samples it keeps."""
import os
import stat
import sys
import time
from datetime import datetime

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _fake_smi(tmp_path, lines):
    data = tmp_path / "samples.csv"
    data.write_text("".join(l + "\n" for l in lines))
    exe = tmp_path / "nvidia-smi"
    exe.write_text(f"#!/bin/sh\ncat '{data}'\nexec sleep 30\n")
    exe.chmod(exe.stat().st_mode | stat.S_IXUSR)
    return str(tmp_path)


def _line(t, sm, reasons=("Not Active",) * 4):
    ts = datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return ", ".join([ts, str(sm), "2070", "900.00", "0x0000000000000000", *reasons])


@pytest.fixture
def path_with(monkeypatch, tmp_path):
    def install(lines):
        monkeypatch.setenv("PATH", _fake_smi(tmp_path, lines) + os.pathsep + os.environ["PATH"])
    return install


def test_samples_inside_the_timed_loop_are_kept(path_with):
    base = time.time() + 100.0
    path_with([_line(base - 10, 1200, ("Active", "Not Active", "Not Active", "Not Active")),
               _line(base + 0.10, 2070), _line(base + 0.15, 2040),
               _line(base + 0.20, 2070, ("Not Active", "Not Active", "Not Active", "Active")),
               _line(base + 10, 900)])
    c = bench.ClockSampler(0)
    time.sleep(0.3)
    c.start(base)
    c.end(base + 0.25)
    ck = c.stop()
    assert ck["samples"] == 3 and ck["window"] == "timed loop"
    assert ck["sm_mhz"] == 2070 and ck["sm_max_mhz"] == 2070
    assert ck["reasons"] == ["sw_power_cap"]


def test_no_sample_inside_falls_back_to_all(path_with):
    base = time.time() + 100.0
    path_with([_line(base - 10, 2070), _line(base + 10, 2060)])
    c = bench.ClockSampler(0)
    time.sleep(0.3)
    c.start(base)
    c.end(base + 0.1)
    ck = c.stop()
    assert ck["samples"] == 2 and ck["window"].startswith("whole sampler run")
    assert ck["sm_mhz"] == 2065


def test_missing_tool_is_reported(monkeypatch, tmp_path):
    monkeypatch.setenv("PATH", str(tmp_path))
    ck = bench.ClockSampler(0).stop()
    assert ck["reasons"] == ["nvidia-smi unavailable"]
