"""Host-side pieces of bench.py that need no GPU: the per-piece roofline
arithmetic and the clock sampler's timed-window filter."""
import datetime
import io
import os

import bench


def test_piece_rooflines_arithmetic():
    n, o = 224, 160
    v = n - o
    peaks = {"hbm_gbs": 6000.0, "bf16_tflops": 2000.0}
    r = bench.piece_rooflines(n, o, ms_eri=20.0, quartets=4e6, ms_ao2mo=10.0, ms_mp2=0.5, peaks=peaks)
    assert r["peak_source"] == "measured"
    assert abs(r["eri"]["quartets_per_s"] - 2e8) < 1.0
    fl = 2.0 * (o * n ** 4 + o * v * n ** 3 + o * o * v * n * n + o * o * v * v * n)
    assert abs(r["ao2mo"]["algorithmic_flop"] - fl) < 1.0
    assert abs(r["ao2mo"]["achieved_tflops"] - fl / 1e-2 / 1e12) < 1e-9
    assert abs(r["ao2mo"]["hbm_frac"] - 8.0 * n ** 4 / 1e-2 / 1e9 / 6000.0) < 1e-12
    assert abs(r["mp2"]["achieved_gbs"] - 8.0 * o * o * v * v / 5e-4 / 1e9) < 1e-6
    # no timings: no entries, and fallback peaks without a peaks file
    r = bench.piece_rooflines(n, o, 0.0, 0.0, 0.0, 0.0, {})
    assert r["peak_source"] == "fallback" and "ao2mo" not in r and "mp2" not in r


class _Done:
    def poll(self):
        return 0


def test_clock_sampler_keeps_the_timed_window():
    c = bench.ClockSampler(0)
    t0 = datetime.datetime(2026, 1, 2, 3, 4, 5)
    rows = []
    for k in range(10):
        t = t0 + datetime.timedelta(milliseconds=200 * k)
        sm = 1200 if k < 3 else 2070
        cap = "Active" if k == 5 else "Not Active"
        rows.append(f"{t.strftime('%Y/%m/%d %H:%M:%S.%f')[:-3]}, 0, {sm}, 2070, 900.0, 0x0, Not Active, "
                    f"Not Active, Not Active, {cap}")
    with open(c.path, "w") as f:
        f.write("\n".join(rows) + "\n")
    try:
        c.proc, c.f = _Done(), io.StringIO()
        # samples 3..6 lie inside the window: idle-clock samples before it are dropped
        c.window(t0 + datetime.timedelta(milliseconds=500), t0 + datetime.timedelta(milliseconds=1300))
        s = c.summary()
        assert s["samples"] == 4 and s["sm_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]
        # a window shorter than the sampling period keeps the nearest sample
        c.window(t0 + datetime.timedelta(milliseconds=410), t0 + datetime.timedelta(milliseconds=420))
        assert c.summary()["samples"] == 1
    finally:
        os.remove(c.path)
