"""Host-side pieces of bench.py that need no GPU: the per-piece roofline
arithmetic and the clock sampler's timed-window filter."""
import datetime
import io
import os

import bench


def _per(**kw):
    base = {k: 0.0 for k in ("fock", "fock_calls", "fock_kernel", "fock_kernel_launches", "eri", "eri_kernel",
                             "quartets", "quartets_f32", "prim_quartets", "diag", "ao2mo", "mp2", "fock_inc_builds",
                             "store_unique", "store_bytes")}
    base.update(kw)
    return base


def test_piece_rooflines_arithmetic():
    n, o = 224, 160
    v = n - o
    peaks = {"hbm_gbs": 6000.0, "bf16_tflops": 2000.0}
    per = _per(eri=25.0, eri_kernel=20.0, quartets=4e6, prim_quartets=1e8, ao2mo=10.0, mp2=0.5, fock_kernel=12.0,
               fock_kernel_launches=12.0, store_unique=5e7, store_bytes=4e8)
    r = bench.piece_rooflines(n, o, per, peaks, 1.25)
    assert r["peak_source"] == "measured" and r["fp64_peak_tflops"] == 1.25
    assert abs(r["eri"]["quartets_per_s"] - 2e8) < 1.0
    # digestion: 6 fma (12 FP64 flops) per unique integral per build of 1 ms
    assert abs(r["fock"]["achieved_tflops"] - 12.0 * 5e7 / 1e-3 / 1e12) < 1e-9
    assert abs(r["fock"]["frac"] - r["fock"]["achieved_tflops"] / 1.25) < 1e-12
    assert abs(r["fock"]["store_gbs"] - 4e8 / 1e-3 / 1e9) < 1e-9
    fl = 2.0 * (o * n ** 4 + o * v * n ** 3 + o * o * v * n * n + o * o * v * v * n)
    assert abs(r["ao2mo"]["algorithmic_flop"] - fl) < 1.0
    assert abs(r["ao2mo"]["achieved_tflops"] - fl / 1e-2 / 1e12) < 1e-9
    assert abs(r["ao2mo"]["hbm_frac"] - 8.0 * n ** 4 / 1e-2 / 1e9 / 6000.0) < 1e-12
    assert abs(r["mp2"]["achieved_gbs"] - 8.0 * o * o * v * v / 5e-4 / 1e9) < 1e-6
    if "achieved_tflops" in r["eri"]:  # with the committed FP64 count per primitive quartet
        f = r["eri"]["fp64_flop_per_prim_quartet"]
        assert abs(r["eri"]["achieved_tflops"] - 1e8 * f / 2e-2 / 1e12) < 1e-9
        top = bench.dominant_roofline(r)
        assert top["bound"] == "fp64" and top["achieved"] == r["eri"]["achieved_tflops"]
    # no timings: no entries, and fallback peaks without a peaks file
    r = bench.piece_rooflines(n, o, _per(), {}, 1.25)
    assert r["peak_source"] == "fallback" and "ao2mo" not in r and "mp2" not in r and "fock" not in r


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


def test_cpu_fit_and_extrapolation():
    """Stage times that grow as N^k in the cluster size N are fitted with
    exponent k and extrapolated exactly; the SCF is iterations x (digestion +
    one DSYGV)."""
    nm = bench.NMOL
    pts = []
    for N in (3, 4, 5, 6):
        pts.append({"nmol": N, "t": {"int1e": 1e-3 * N ** 2, "int2e": 1e-4 * N ** 3.5, "fock": 1e-5 * N ** 4,
                                     "ao2mo": 1e-6 * N ** 5, "mp2": 1e-7 * N ** 4}})
    fit, ext = bench.fit_and_extrapolate(pts, 10, 0.02)
    assert abs(fit["int2e"]["exponent"] - 3.5) < 1e-9 and abs(fit["ao2mo"]["exponent"] - 5.0) < 1e-9
    expect = {"int1e": 1e-3 * nm ** 2, "int2e": 1e-4 * nm ** 3.5, "scf": 10 * (1e-5 * nm ** 4 + 0.02),
              "ao2mo": 1e-6 * nm ** 5, "mp2": 1e-7 * nm ** 4}
    assert all(abs(ext[k] - v) <= 1e-9 * v for k, v in expect.items()), ext


def test_cpu_digestion_from_the_large_order_point():
    pts = [{"nmol": N, "t": {"int1e": 1.0, "int2e": 1.0, "fock": 1e-5 * N ** 5, "ao2mo": 1.0, "mp2": 1.0}}
           for N in (3, 4, 5, 6)]
    nm = bench.NMOL
    fit, ext = bench.fit_and_extrapolate(pts, 2, 0.5, (84, 0.4))
    assert abs(ext["scf"] - 2 * (0.4 * (7.0 * nm / 84) ** 4 + 0.5)) < 1e-9
    assert fit["fock"]["large_order_point_s"] == [84, 0.4]
