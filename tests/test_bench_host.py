"""Host-side logic of bench.py that needs no GPU: the clock sampler (against a
stand-in nvidia-smi that writes samples on a timer) and the packet sampler of
the CPU baseline."""
import os
import stat
import sys
import time

import numpy as np

import bench

FAKE_SMI = """#!{python}
import sys, time
path = sys.argv[sys.argv.index("-f") + 1]
time.sleep(0.15)
i = 0
while True:
    with open(path, "a") as h:
        # the first sample idles at 1000 MHz, the later ones run at 2070 MHz
        h.write("0, %d, 2070, 500.0, 0x0, Not Active, Not Active, Not Active, %s\\n"
                % (1000 if i == 0 else 2070, "Active" if i == 2 else "Not Active"))
    i += 1
    time.sleep(0.05)
"""


def test_clock_sampler_drops_samples_before_the_timed_region(tmp_path, monkeypatch):
    smi = tmp_path / "nvidia-smi"
    smi.write_text(FAKE_SMI.format(python=sys.executable))
    smi.chmod(smi.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    with bench.ClockSampler(0) as clk:
        assert clk.before >= 1  # the sampler was running before the region
        time.sleep(0.3)
    s = clk.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["samples"] >= 2
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.summary()["sm_mhz"] is None


def test_sample_packets_spans_the_frame():
    rays = np.arange(10 * 256 + 17, dtype=np.float32)[:, None].repeat(8, 1)
    s = bench.sample_packets(rays, 0.2)
    # every 5th packet of 256 rays: packets 0, 5 and the ragged last one (17 rays)
    first = s[:, 0].astype(np.int64)
    assert first[0] == 0 and first[256] == 5 * 256 and first[512] == 10 * 256
    assert s.shape[0] == 2 * 256 + 17
    assert np.array_equal(bench.sample_packets(rays, 1.0), rays)
