"""The reference arm of bench.py on the CPU: `--impl reference` times the
FP64 oracle on the bench workload and prints the one JSON line the
benchmark contract asks for, on the same metric, unit and config as the
GPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, out.stdout
    line = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "pose-evals/s"
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 3 and line["higher_is_better"] is True
    assert "3 bones" in line["config"]["workload"] and line["config"]["particles"] == 100
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"] and cb["value"] == line["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": "pose-evals/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
