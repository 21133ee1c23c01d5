"""bench.py's clock record: only nvidia-smi samples taken inside the timed region count (CPU, no GPU needed)."""
import datetime
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


class _Done:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _row(ts, mhz, hw="Not Active", cap="Not Active"):
    return "0, %d, 2070, 900.0, 0x0, %s, Not Active, Not Active, %s, %s\n" % (
        mhz, hw, cap, ts.strftime("%Y/%m/%d %H:%M:%S.%f")[:-3])


def _stop(tmp_path, rows, window):
    c = bench.Clocks(0, path=str(tmp_path / "clocks.csv"))
    with open(c.path, "w") as fh:
        fh.writelines(rows)
    c.f = open(c.path, "a")
    c.proc = _Done()
    return c.stop(window)


def test_samples_outside_the_timed_region_are_ignored(tmp_path):
    t0 = datetime.datetime(2026, 1, 1, 12, 0, 0)
    rows = [_row(t0 - datetime.timedelta(seconds=2), 1200, hw="Active"),   # warm-up: slowed, outside
            _row(t0 + datetime.timedelta(milliseconds=100), 2070),
            _row(t0 + datetime.timedelta(milliseconds=150), 2055, cap="Active"),
            _row(t0 + datetime.timedelta(milliseconds=200), 2070),
            _row(t0 + datetime.timedelta(seconds=5), 900)]                   # after the region
    r = _stop(tmp_path, rows, (t0, t0 + datetime.timedelta(seconds=1)))
    assert r["samples_in_timed_region"] == 3 and r["samples"] == 3
    assert r["sm_mhz"] == 2070 and r["sm_max_mhz"] == 2070
    assert r["reasons"] == ["sw_power_cap"]


def test_all_samples_are_used_when_none_falls_inside(tmp_path):
    t0 = datetime.datetime(2026, 1, 1, 12, 0, 0)
    rows = [_row(t0 - datetime.timedelta(seconds=1), 2000), "garbage line\n",
            _row(t0 + datetime.timedelta(seconds=3), 2070, hw="Active")]
    r = _stop(tmp_path, rows, (t0, t0 + datetime.timedelta(milliseconds=10)))
    assert r["samples_in_timed_region"] == 0 and r["samples"] == 2
    assert r["reasons"] == ["hw_slowdown"]
