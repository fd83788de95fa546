"""Host logic of bench.py that needs no GPU: the clock record keeps only the samples taken
inside the timed region (by nvidia-smi's own timestamps) and collects the throttle reasons
seen there; the roofline's DRAM traffic comes from the committed Gram-kernel profile."""
import datetime
import os
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


class _Done:
    """Stands in for the finished nvidia-smi process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _line(ts, clk, reasons=("Not Active",) * 4):
    return ", ".join([ts.strftime("%Y/%m/%d %H:%M:%S.%f")[:-3], str(clk), "2070", "850.12", "0x0000000000000000",
                      *reasons])


def test_clock_record_keeps_the_timed_region_only():
    s = bench.ClockSampler(0)
    s.proc = _Done()
    t0 = datetime.datetime(2026, 1, 2, 3, 4, 5, 0)
    s.t0, s.t1 = t0, t0 + datetime.timedelta(milliseconds=100)
    ms = lambda k: t0 + datetime.timedelta(milliseconds=k)  # noqa: E731
    s.lines = [
        _line(ms(-50), 1200, ("Active", "Not Active", "Not Active", "Not Active")),  # warm-up, throttled
        _line(ms(10), 2070),
        _line(ms(35), 2055, ("Not Active", "Not Active", "Not Active", "Active")),  # power cap inside
        _line(ms(60), 2070),
        "garbage line",
        _line(ms(150), 900, ("Not Active", "Active", "Not Active", "Not Active")),  # after the region
    ]
    rec = s.stop()
    assert rec["samples"] == 3 and rec["samples_all"] == 5
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"]  # the hw_slowdown before and the thermal one after are not in it


def test_clock_record_without_nvidia_smi():
    s = bench.ClockSampler(0)
    rec = s.stop()
    assert rec["sm_mhz"] is None and rec["reasons"] == ["nvidia-smi unavailable"]


def test_roofline_traffic_from_the_committed_profile():
    t = bench.read_profile_traffic()
    assert t is not None and t > 0
    with open(os.path.join(ROOT, "profiles", "k_gram_bf16__k2_1Mx128.md")) as f:
        lines = [ln for ln in f if ln.startswith("dram_bytes_per_launch:")]
    assert len(lines) == 1 and float(lines[0].split(":")[1]) == t
