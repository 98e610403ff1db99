"""bench.py's clock record (CPU, with a stand-in nvidia-smi on PATH that
prints the queried columns every interval): the sampler is running before
the timed region starts, keeps only the rows written from the region's
start, and reads the throttle reasons."""
import os
import sys
import time

FAKE = """\
#!{python}
import sys, time
ms = int(sys.argv[sys.argv.index("-lms") + 1])
time.sleep(0.15)  # the tool's start-up
while True:
    v = open({mhz!r}).read().strip()
    cap = "Active" if v == "1500" else "Not Active"
    print("0, " + v + ", 2070, 500.00, 0x0000000000000000, Not Active, Not Active, Not Active, " + cap,
          flush=True)
    time.sleep(ms / 1000)
"""


def _fake(tmp_path, monkeypatch, mhz_value):
    mhz = tmp_path / "mhz"
    mhz.write_text(mhz_value)
    tool = tmp_path / "nvidia-smi"
    tool.write_text(FAKE.format(python=sys.executable, mhz=str(mhz)))
    tool.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    return mhz


def test_rows_before_the_region_are_dropped(tmp_path, monkeypatch):
    import bench
    mhz = _fake(tmp_path, monkeypatch, "1000")
    clk = bench.Clocks(0, interval_ms=10)
    assert clk._rows() >= 1  # the constructor waited for the first row
    time.sleep(0.05)
    mhz.write_text("2070")
    time.sleep(0.05)
    clk.mark()
    time.sleep(0.1)
    out = clk.stop()
    assert out["samples"] >= 3, out
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["reasons"] == [], out


def test_a_region_shorter_than_the_interval_still_gets_a_row(tmp_path, monkeypatch):
    import bench
    mhz = _fake(tmp_path, monkeypatch, "1500")
    clk = bench.Clocks(0, interval_ms=100)
    clk.mark()
    out = clk.stop()  # at once: waits for the next row
    assert out["samples"] >= 1, out
    assert out["sm_mhz"] == 1500.0 and out["reasons"] == ["sw_power_cap"], out
    assert mhz.exists()


def test_no_tool_no_clocks(tmp_path, monkeypatch):
    import bench
    monkeypatch.setenv("PATH", str(tmp_path))
    clk = bench.Clocks(0)
    clk.mark()
    out = clk.stop()
    assert out["sm_mhz"] is None and out["samples"] == 0 and out["reasons"] == ["nvidia-smi unavailable"]
