"""The reference arm of bench.py on the CPU: one JSON line with the metric,
unit and configuration of the GPU arm, `impl: "reference"`, a cpu_baseline
describing the run and an e2e block without host-device copies."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--ref-rays", "20000"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "traced rays/s" and d["unit"] == "rays/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1
    # the GPU arm's configuration; the CPU times a sample of each step's rays
    assert d["config"]["workload"] == "hole_triangles" and d["config"]["n_rays_per_step"] == 10_000_000
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["sample_rays_per_step"] == 20000
    assert d["e2e"] == {"value": d["value"], "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
