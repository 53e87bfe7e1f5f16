"""bench.py's one-line JSON contract, on small cases: the reference arm (the CPU
oracle) here, the GPU arm on a GB300."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config"}


def run_bench(*args, timeout=600):
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                       text=True, timeout=timeout)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, p.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    d = run_bench("--impl", "reference", "--n", "6", "--steps", "2", "--warmup", "1")
    assert BASE_KEYS <= d.keys()
    assert d["impl"] == "reference" and d["unit"] == "atom-steps/s" and d["value"] > 0
    assert d["n_gpus"] == 1 and d["steps"] == 2 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= cb.keys() and cb["value"] == d["value"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("lj_fcc_6^3")


@pytest.mark.gpu
def test_gpu_arm_line():
    d = run_bench("--n", "12", "--steps", "5", "--warmup", "3")
    assert BASE_KEYS <= d.keys() and "impl" not in d
    assert d["value"] > 0 and d["unit"] == "atom-steps/s" and d["n_gpus"] == 1 and d["scaling"] == "weak"
    assert d["vs_baseline"] is None and d["data"] == "synthetic"
    rf = d["roofline"]
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= rf.keys()
    assert rf["achieved"] > 0 and rf["peak"] > 0 and abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-9
    cb = d["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= cb.keys() and cb["value"] > 0
    e = d["e2e"]
    assert {"value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"} <= e.keys()
    assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= d["clocks"].keys()
    ph = d["phases"]
    assert ph["force_only_mixed"]["ms"] > 0 and ph["neighbour_build_ms_per_rebuild"] > 0
    assert d["force_error_mixed_vs_fp64"]["max"] <= 1e-5
