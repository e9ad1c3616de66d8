"""CPU tests of the bench's clock sampling summary: only samples inside the timed window count, the
throttle reasons seen there are reported, and a window shorter than the sampling interval falls back to
the nearest sample (fake nvidia-smi output, no GPU)."""

import datetime
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _sampler(tmp_path, rows):
    import bench

    cs = bench.ClockSampler(0)
    cs.path = str(tmp_path / "clocks.csv")
    with open(cs.path, "w") as f:
        for t, mhz, reason in rows:
            flags = ["Not Active"] * 4
            if reason is not None:
                flags[reason] = "Active"
            f.write(f"{t.strftime('%Y/%m/%d %H:%M:%S.%f')[:-3]}, 0, {mhz}, 2070, 900.00, 0x0, " + ", ".join(flags) + "\n")
    cs.proc = object()  # as if nvidia-smi had been started
    return cs


def test_summary_keeps_only_the_timed_window(tmp_path):
    t0 = datetime.datetime(2026, 1, 1, 12, 0, 0)
    ms = lambda k: t0 + datetime.timedelta(milliseconds=50 * k)  # noqa: E731
    rows = [(ms(k), 1500, 0) for k in range(4)]                     # warm-up: slowed, hw_slowdown
    rows += [(ms(k), 2070, None) for k in range(10, 16)]            # the timed window
    rows += [(ms(k), 1800, 3) for k in range(30, 33)]               # afterwards: power cap
    cs = _sampler(tmp_path, rows)
    cs.mark(ms(10), ms(15))
    s = cs.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == [] and s["samples"] == 6


def test_summary_reports_reasons_seen_in_the_window(tmp_path):
    t0 = datetime.datetime(2026, 1, 1, 12, 0, 0)
    ms = lambda k: t0 + datetime.timedelta(milliseconds=50 * k)  # noqa: E731
    rows = [(ms(k), 2070, None) for k in range(5)] + [(ms(5), 1900, 3), (ms(6), 1700, 1)]
    cs = _sampler(tmp_path, rows)
    cs.mark(ms(0), ms(6))
    s = cs.summary()
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert s["samples"] == 7


def test_short_window_uses_the_nearest_sample(tmp_path):
    t0 = datetime.datetime(2026, 1, 1, 12, 0, 0)
    rows = [(t0, 2070, None), (t0 + datetime.timedelta(seconds=1), 1200, 0)]
    cs = _sampler(tmp_path, rows)
    w = t0 + datetime.timedelta(milliseconds=200)
    cs.mark(w, w + datetime.timedelta(milliseconds=5))
    s = cs.summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 2070.0 and s["reasons"] == []
