"""Host logic of bench.py that needs no GPU: the clock summary (samples kept to
the timed region by their own timestamps, the fallback span, throttle
reasons, the busiest GPU) and the algorithmic byte model."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Proc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _row(ts, gpu, sm, power, hw="Not Active", cap="Not Active"):
    # timestamp, index, clocks.sm, clocks.max.sm, power.draw, active, hw, hw_thermal, sw_thermal, sw_power_cap
    return [ts, gpu, str(sm), "2070", str(power), "0x0", hw, "Not Active", "Not Active", cap]


def test_clock_summary_keeps_the_timed_region():
    b = _bench()
    s = b.ClockSampler()
    s.proc = _Proc()
    s.rows = [_row(9.0, "0", 1000, 150.0),                      # idle, before the region
              _row(10.1, "0", 2070, 900.0), _row(10.2, "0", 2055, 950.0, cap="Active"),
              _row(10.3, "0", 2070, 940.0),
              _row(10.1, "1", 345, 90.0),                        # another, idle GPU
              _row(11.5, "0", 1200, 200.0, hw="Active")]         # after the region
    out = s.stop((10.0, 10.4), (10.0, 12.0))
    assert out["gpu"] == "0" and out["samples"] == 3 and out["span"] == "timed region"
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_summary_falls_back_to_the_loaded_span():
    b = _bench()
    s = b.ClockSampler()
    s.proc = _Proc()
    s.rows = [_row(9.0, "0", 1000, 150.0), _row(10.6, "0", 2070, 900.0, hw="Active")]
    out = s.stop((10.0, 10.05), (10.0, 11.0))
    assert out["samples"] == 1 and out["span"].startswith("timed region and")
    assert out["reasons"] == ["hw_slowdown"]
    s2 = b.ClockSampler()
    s2.proc = _Proc()
    s2.rows = [_row(9.0, "0", 1000, 150.0)]
    assert s2.stop((10.0, 10.05), (10.0, 11.0)) is None


def test_byte_model():
    b = _bench()
    nb, px, rpx = 1000, 640 * 480, 640 * 480
    assert b.bytes_per_launch("integrate", nb, px, rpx, 0) == nb * 512 * 32 + px * 8
    assert b.bytes_per_launch("raycast", nb, px, rpx, 0) == nb * (512 * 4 + 16) + rpx * 36
    assert b.bytes_per_launch("collect", nb, px, rpx, 0) == nb * 32
    assert b.bytes_per_launch("unknown", nb, px, rpx, 0) == 0.0
