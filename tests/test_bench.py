"""bench.py's reference arm (the FP32 oracle port of the reference's
routines on the host cores) on a small workload, and its one JSON line: no
GPU needed."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    cmd = [sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--width", "96", "--height", "54",
           "--lights", "32", "--triangles", "500", "--steps", "3", "--warmup", "3", "--cpu-seconds", "0.2"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [line for line in out.stdout.splitlines() if line.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Gsamples/s" and d["value"] > 0
    assert (d["steps"], d["warmup"], d["n_gpus"], d["higher_is_better"]) == (3, 3, 1, True)
    assert d["metric"].startswith("Gsamples/s (shadowed single frame: 96x54 fBm heightfield, 32 polygon lights")
    assert d["vs_baseline"] is None
    cpu = d["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == d["value"] and cpu["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
