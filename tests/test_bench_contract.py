"""The JSON line of bench.py's reference arm (the oracle's FP64 CGNE on the host cores), on a small
lattice: the keys the measurement contract needs, and the same workload string as the GPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                          "--dims", "4,4,4,8"], cwd=ROOT, capture_output=True, text=True, check=True).stdout
    line = json.loads([ln for ln in out.splitlines() if ln.startswith("{")][-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "s"
    assert line["higher_is_better"] is False and line["value"] > 0
    assert line["config"]["workload"] == bench.workload_desc((4, 4, 4, 8))
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_workload_string_names_the_run():
    w = bench.workload_desc(bench.DIMS)
    assert w.startswith("32x32x32x64 ") and f"kappa={bench.KAPPA}" in w and f"FP64 true residual {bench.RSD}" in w
