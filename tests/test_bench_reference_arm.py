"""The reference arm of bench.py (`--impl reference`) on the CPU: it prints
one JSON line with the GPU arm's metric, unit and config for the same
arguments, its own CPU baseline description, and an e2e of the same value
with no host-device bytes; the decoded output is checked against the
source symbols."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    sys.path.insert(0, ROOT)
    import bench

    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--mb", "2",
           "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "GB/s"
    assert line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["value"] > 0 and line["bit_exact"] is True
    cfg = line["config"]
    assert cfg["workload"] == "plain 2MiB lambda=0.05 L=1024"
    assert set(cfg) == {"workload", "n_symbols", "n_units", "lambda", "L", "seed"}
    assert cfg["n_symbols"] == 2 << 20
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "GB/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
