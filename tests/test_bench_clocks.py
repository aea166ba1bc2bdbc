"""bench.py's clock record: samples outside the timed window are dropped,
throttle reasons inside it are reported, and a run without samples inside
the window says so. nvidia-smi is replaced by a CSV file written here."""
import datetime
import importlib.util
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["bench_under_test"] = mod
    spec.loader.exec_module(mod)
    return mod


class _Done:
    def terminate(self): pass
    def wait(self, timeout=None): return 0
    def kill(self): pass


def sampler_with(tmp_path, rows, t0, t1):
    bench = load_bench()
    s = bench.ClockSampler(0)
    s.path = str(tmp_path / "clocks.csv")
    with open(s.path, "w") as f:
        for ts, mhz, reasons in rows:
            act = ["Active" if r in reasons else "Not Active"
                   for r in ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")]
            f.write(", ".join([ts.strftime("%Y/%m/%d %H:%M:%S.%f")[:-3], "0", str(mhz), "2070", "900.0", "0x0"] + act)
                    + "\n")
    s.proc = _Done()
    s.t0, s.t1 = t0, t1
    return s


def test_only_samples_inside_the_window_count(tmp_path):
    t = datetime.datetime(2026, 1, 1, 12, 0, 0)
    ms = lambda k: t + datetime.timedelta(milliseconds=k)   # noqa: E731
    rows = [(ms(0), 1200.0, {"hw_slowdown"}),                # warm-up, before the window
            (ms(500), 2070.0, set()), (ms(550), 2070.0, {"sw_power_cap"}), (ms(600), 2055.0, set()),
            (ms(1500), 900.0, {"sw_thermal_slowdown"})]      # after the window
    out = sampler_with(tmp_path, rows, ms(480), ms(620)).stop()
    assert out["samples"] == 3
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
    assert "note" not in out


def test_no_sample_inside_the_window_is_reported(tmp_path):
    t = datetime.datetime(2026, 1, 1, 12, 0, 0)
    rows = [(t, 2070.0, set()), (t + datetime.timedelta(seconds=2), 2070.0, set())]
    out = sampler_with(tmp_path, rows, t + datetime.timedelta(milliseconds=900),
                       t + datetime.timedelta(milliseconds=950)).stop()
    assert out["samples"] == 2 and "note" in out
