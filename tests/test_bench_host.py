"""bench.py's host side (no GPU): the clock-sample summary that decides
whether a run saw a throttle reason, and the reference arm's JSON line."""
import importlib.util
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_summary_reports_throttle_reasons():
    cs = _bench().ClockSampler()
    assert cs.summary()["reasons"] == ["unsampled"]
    na = "Not Active"
    cs.rows = [["0", "2070", "2070", "900.1", "0x0", na, na, na, na],
               ["0", "1980", "2070", "1400.0", "0x4", na, na, na, "Active"],
               ["0", "2070", "2070", "1390.5", "0x0", na, na, na, na]]
    s = cs.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    cs.rows.append(["0", "1500", "2070", "1000", "0x8", "Active", na, "Active", na])
    assert cs.summary()["reasons"] == ["hw_slowdown", "sw_power_cap", "sw_thermal_slowdown"]
    # rows that are not numbers (a header, an error line) are skipped
    cs.rows = [["index", "clocks.sm [MHz]"], ["0", "[N/A]", "2070", "1", "0x0", na, na, na, na]]
    s = cs.summary()
    assert s["sm_mhz"] is None and s["reasons"] == []


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference`: the CPU restatement on the host cores, one
    JSON line with the keys the contract names."""
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "solves/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["batch_per_gpu"] == 8192
