"""bench.py's CPU-side pieces: the reference arm's JSON line (the oracle port on the host
cores) and the clock-sample summary that flags throttled runs."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--m", "400"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "Gaussian matvec Gpairs/s" and d["unit"] == "Gpairs/s"
    assert d["value"] > 0 and d["steps"] == 1 and d["higher_is_better"] is True
    # the same workload as the GPU arm: every point of the m x m lattice, not a sample
    assert d["config"]["workload"] == "2d_lamb_oseen_m400" and d["config"]["n_points"] == 400 * 400
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Gpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_clock_summary_reports_throttle_reasons():
    sys.path.insert(0, ROOT)
    import bench
    c = bench.Clocks(0)
    c.rows = [["2070", "2070", "Not Active", "Not Active", "Not Active", "Not Active"],
              ["1980", "2070", "Not Active", "Not Active", "Not Active", "Active"],
              ["2010", "2070", "Active", "Not Active", "Not Active", "Not Active"]]
    s = c.summary()
    assert s["sm_mhz"] == 2010.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert bench.Clocks(0).summary()["reasons"] == ["unsampled"]


def test_hbm_view_of_the_matvec():
    sys.path.insert(0, ROOT)
    import bench
    v = bench.hbm_view(32 * 4_000_000, 44.8)
    assert v["bound"] == "hbm" and v["unit"] == "GB/s" and v["bytes_per_launch"] == 128_000_000
    assert abs(v["achieved"] - 128e6 / 44.8e-3 / 1e9) < 1e-9
    assert v["peak"] > 0 and abs(v["frac"] - v["achieved"] / v["peak"]) < 1e-12


def test_host_core_solve_child_small(tmp_path):
    """The child process that solves the 4x10^6-point problem on the host cores (memory
    guard, address-space cap, weights file), here on a 3600-point lattice."""
    out = str(tmp_path / "cpu.json")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--cpu-solve-child", out, "--m", "60",
                        "--seed", "5"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.load(open(out))
    assert d["status"] == "ok" and d["reason"] == 2 and d["its"] > 0 and d["setup_status"] == 0
    import numpy as np
    g = np.load(out + ".g.npy")
    assert g.shape == (3600,) and np.all(np.isfinite(g))
