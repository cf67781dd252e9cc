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
           "--lights", "32", "--clusters", "8", "--triangles", "500", "--steps", "3", "--warmup", "3", "--cpu-seconds", "0.2"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [line for line in out.stdout.splitlines() if line.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Gsamples/s" and d["value"] > 0
    assert (d["steps"], d["warmup"], d["n_gpus"], d["higher_is_better"]) == (3, 3, 1, True)
    assert d["metric"].startswith("Gsamples/s (many-lights frame: 96x54 fBm heightfield, 32 polygon lights (3-8 "
                                  "vertices) in 8 k-means clusters")
    assert d["vs_baseline"] is None
    cpu = d["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == d["value"] and cpu["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_default_workload_is_the_headline_configuration():
    """With no flags the bench runs the configuration the headline metric is
    quoted on: 1080p, 16,384 lights in 256 clusters, 1M occluders, M = 32."""
    sys.path.insert(0, REPO)
    import bench
    a = bench.parse([])
    assert (a.workload, a.width, a.height, a.lights, a.clusters, a.triangles, a.candidates, a.spp) == (
        "headline", 1920, 1080, 16384, 256, 1_000_000, 32, 4)
    assert bench.is_headline(a) and bench.metric_name(a) == bench.HEADLINE_METRIC
    b = bench.parse(["--workload", "throughput"])
    assert (b.lights, b.triangles, b.clusters) == (1024, 200_000, 0)


def test_reference_arm_under_two_ranks_prints_once():
    """Launched as the multi-GPU bench is (torchrun, two ranks), the reference
    arm runs on rank 0 alone: one JSON line in all, and every rank exits 0."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29531", os.path.join(REPO, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--width", "64", "--height", "36", "--lights", "16",
           "--clusters", "4", "--triangles", "200", "--steps", "3", "--warmup", "3", "--cpu-seconds", "0.1"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [line for line in out.stdout.splitlines() if line.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
