"""Host-side pieces of bench.py that shape its JSON line, checked without a GPU: the clock summary
(median SM clock under load, throttle reasons seen inside the timed region only) and the graph
fallback's bookkeeping."""

import bench


def _row(sm, mx, **active):
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    flags = ["Active" if active.get(n) else "Not Active" for n in names]
    return ["0", str(sm), str(mx), "900.0", "0x0", *flags]


def test_clock_summary_uses_the_timed_region_only():
    c = bench.Clocks(0)
    c.t0, c.t1 = 10.0, 20.0
    c.rows = [(9.0, _row(500, 2070, hw_thermal_slowdown=True)),  # before the region: ignored
              (11.0, _row(2000, 2070)), (12.0, _row(2070, 2070, sw_power_cap=True)), (13.0, _row(1900, 2070)),
              (25.0, _row(600, 2070, hw_slowdown=True))]  # after the region: ignored
    s = c.summary()
    assert s["sm_mhz"] == 2000.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["samples"] == 3


def test_clock_summary_without_samples():
    c = bench.Clocks(0)
    c.t0, c.t1 = 1.0, 2.0
    assert c.summary()["reasons"] == ["unsampled"]


def test_graph_source_names_the_fallback():
    saved = dict(bench._BUILT)
    try:
        bench._BUILT.clear()
        assert "reference's CPU builder" in bench.graph_source()
        bench._BUILT.update(path="/tmp/x.glass", seconds=3.0)
        assert "GPU builder" in bench.graph_source() and "absent" in bench.graph_source()
        bench._BUILT["stale"] = True
        assert "differ" in bench.graph_source()
    finally:
        bench._BUILT.clear()
        bench._BUILT.update(saved)


def test_cpu_legs_load_no_library_of_the_package(tmp_path):
    """The reference arm and the CPU baseline search through the oracle's own graph readers, so the
    process maps the oracle's library and none of this package's (checked in a child process on the
    golden graph's NSG-format twin)."""
    import os
    import shutil
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "g.glass"
    shutil.copy(os.path.join(root, "tests", "golden", "nsg_d100.glass"), src)
    from oracle import compact_graphs

    twin = compact_graphs.compact(str(src))
    code = f"""
import sys
sys.path.insert(0, {root!r})
import bench
from tests.golden import spec
bench.graph_file = lambda: ({twin!r}, "nsg")
cb, s, ids = bench.cpu_baseline(spec.base(), spec.queries(), 32, 50)
assert ids.shape == (50, 10) and (ids >= 0).all()
maps = open("/proc/self/maps").read()
assert "libglass_oracle.so" in maps
assert "libglass_gb300" not in maps and "_glass" not in maps, "package library mapped"
print("ok")
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr


def test_profiling_cases_are_declared(monkeypatch):
    """bench.py --case NAME runs one small case of the other kernels for ncu captures; every case
    the help text names has a runner, and --tuning parses as five integers."""
    import sys

    assert {"setdata", "lowrank-e5m2", "lowrank-sq8u", "sphere-sq4u-ip"} <= set(bench.CASES)
    for what, run in bench.CASES.values():
        assert isinstance(what, str) and callable(run)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--profile", "--tuning", "2,1,1,2,13", "--case", "setdata"])
    a = bench.args_()
    assert a.case == "setdata" and [int(x) for x in a.tuning.split(",")] == [2, 1, 1, 2, 13]
