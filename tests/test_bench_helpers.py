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


def test_threshold_flags():
    a = bench.parse_args([])
    assert a.eri_f32_tau == bench.ERI_F32_TAU and a.fock_inc_tau == bench.FOCK_INC_TAU
    assert 0.0 <= bench.FOCK_INC_TAU <= 1e-2 and bench.ERI_F32_TAU >= 0.0
    a = bench.parse_args(["--eri-f32-tau", "3e-5", "--fock-inc-tau", "1e-3", "--warmup", "1"])
    assert (a.eri_f32_tau, a.fock_inc_tau, a.warmup) == (3e-5, 1e-3, 3)  # at least 3 warm-up steps
    for bad in (["--fock-inc-tau", "0.02"], ["--fock-inc-tau", "-1e-3"], ["--eri-f32-tau", "-1"]):
        try:
            bench.parse_args(bad)
        except SystemExit as e:
            assert e.code == 2
        else:
            raise AssertionError(bad)


def test_cpu_extrapolation_by_loop_counts():
    """A sample of the cluster itself extrapolates to its own times (x iterations
    for the Fock digestion); one of half the waters scales by the loop counts."""
    nm = bench.NMOL
    t = {"int1e": 1.0, "int2e": 2.0, "fock": 3.0, "ao2mo": 4.0, "mp2": 5.0}
    s = {"n": 7 * nm, "nset": 12 * nm, "nnuc": 3 * nm, "no": 5 * nm, "t": t}
    r = bench._extrapolate(s, 25)
    assert r == {"int1e": 1.0, "int2e": 2.0, "scf": 75.0, "ao2mo": 4.0, "mp2": 5.0}
    h = nm // 2
    s = {"n": 7 * h, "nset": 12 * h, "nnuc": 3 * h, "no": 5 * h, "t": t}
    r = bench._extrapolate(s, 1)
    f = nm / h
    expect = {"int1e": f ** 3, "int2e": 2.0 * f ** 4, "scf": 3.0 * f ** 4, "ao2mo": 4.0 * f ** 5,
              "mp2": 5.0 * f ** 4}
    assert all(abs(r[k] - v) <= 1e-12 * v for k, v in expect.items()), r
