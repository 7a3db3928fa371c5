"""The GPU arm of bench.py: one JSON line carrying the fields of the benchmark
contract -- metric, value, timing, configuration, the roofline of the path
kernel, the CPU baseline, the end-to-end number with its host-device bytes,
the kernel-launch count and the clocks sampled during the timed region."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_json_line():
    cmd = [sys.executable, "bench.py", "--steps", "3", "--warmup", "3", "--e2e-steps", "1", "--cpu-rays", "20000",
           "--no-batch", "--no-plain", "--no-adjoint", "--no-rough", "--no-one-pct"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["metric"] == "traced rays/s" and d["unit"] == "rays/s" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3 and d["scaling"] == "weak"
    assert d["value"] > 0 and abs(d["value"] * d["ms_per_step"] / 1e3 - d["config"]["n_rays_per_step"]) < \
        1e-6 * d["config"]["n_rays_per_step"]
    assert d["config"]["workload"] == "hole_triangles" and d["config"]["n_rays_per_step"] == 10_000_000
    roof = d["roofline"]
    assert roof["bound"] in ("hbm", "tensor") and roof["unit"] == "GB/s"
    assert roof["achieved"] > 0 and roof["peak"] > 0 and abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-9
    assert roof["traffic"] is None or roof["traffic"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["unit"] == "rays/s"
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0
    assert set(d["clocks"]) >= {"sm_mhz", "sm_max_mhz", "reasons"}
