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


def test_roofline_arithmetic_of_the_bench_line():
    """The bench line's per-kernel table and roofline from given CUDA-event
    times and op counts: achieved = FLOP per pixel-sample x pixel-samples per
    launch / launch time, frac = achieved / peak, the dominant kernel the
    slowest, DRAM traffic scaled from the captured launch's pixel-samples."""
    sys.path.insert(0, REPO)
    import bench
    calls = 4
    prof = {"calls": calls, "candidates": 4 * 14.0, "shade": 4 * 3.5, "ray_sort": 4 * 0.5, "shadow_trace": 4 * 5.0,
            "resolve": 4 * 0.25}
    info = {"flops_per_sample": 26000.0, "candidate_flops_per_sample": 23000.0, "shade_flops_per_sample": 3000.0,
            "trace_flops_per_sample": 1500.0, "trace_bytes_per_sample": 2800.0}
    samples = 8_294_400
    peak = 80.0
    k = bench.kernel_table(prof, samples, info, peak, {})
    cand = k["ris_candidates_binned_kernel"]
    assert cand["ms_per_launch"] == 14.0
    want = 23000.0 * samples / 14e-3 / 1e12
    assert abs(cand["achieved_tflops"] - want) <= 1e-9 * want and abs(cand["frac"] - want / peak) <= 1e-12
    tr = k["shadow_trace_kernel"]
    assert abs(tr["node_triangle_gbs"] - 2800.0 * samples / 5e-3 / 1e9) <= 1e-6
    assert k["ris_resolve_kernel"]["achieved_tflops"] == 0.0
    bench.attach_dram(k, "many_lights_1080p", samples, {"hbm_gbs": 7000.0})
    with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
        t = json.load(f)["many_lights_1080p"]["ris_candidates_binned_kernel"]
    dram = t["dram_bytes"] * samples / t["pixel_samples"]
    assert abs(cand["dram_bytes_per_launch"] - dram) <= 1e-6 * dram
    assert abs(cand["dram_frac_of_hbm"] - dram / 14e-3 / 1e9 / 7000.0) <= 1e-12
    ms_step = 23.25
    r = bench.roofline_of(k, peak, info["flops_per_sample"], samples, ms_step, 152, 2070.0, "many_lights_1080p")
    assert r["kernel"] == "ris_candidates_binned_kernel" and r["unit"] == "TFLOP/s" and r["peak"] == peak
    assert r["achieved"] == cand["achieved_tflops"] and r["frac"] == cand["frac"]
    assert abs(r["frac"] - r["achieved"] / r["peak"]) <= 1e-12
    assert abs(r["traffic"] - dram) <= 1e-6 * dram
    assert abs(r["whole_step_frac"] - 26000.0 * samples / (ms_step / 1e3) / 1e12 / peak) <= 1e-12
    a = bench.parse([])
    rates = bench.rates_of(a, {"value": 0.35, "ms_per_step": ms_step, "rays_per_step": 16_000_000}, k)
    assert abs(rates["gcandidates_per_s"] - 0.35 * 32) <= 1e-12
    assert abs(rates["grays_per_s_trace_kernel"] - 16e6 / 5e-3 / 1e9) <= 1e-9
    assert bench.rates_of(a, {"value": 0.35, "ms_per_step": ms_step}, k)["grays_per_s_step"] is None
