"""Benchmark of the shading path on the shadowed single-frame workload.

Workload: a 1920x1080 G-buffer of a seeded fBm heightfield, 1024 convex
polygon lights with 3..8 vertices (areas log-uniform [0.01, 1]), 200k random
occluder triangles (edge 0.05..0.5) in [-6, 6]^2 x [0, 2] behind a SAH BVH,
plain LTC-RIS with M = 32 candidates, 4 samples per pixel.  One step shades
one frame (4 spp) in one kernel launch.  Metric: pixel-samples per second
(one sample = M candidates + the PSA/MIS shade with its shadow rays).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Prints one JSON line (rank 0).  N > 1 runs one process per GPU (torchrun),
each shading its own frame (weak scaling, no data-path collective).
"""
import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

def count_name(n):
    """200000 -> '200k'; counts that are not whole thousands as they are."""
    return "%dk" % (n // 1000) if n >= 1000 and n % 1000 == 0 else str(n)


def workload_name(a):
    if a.scene == "plane":
        return ("plane of quads: %dx%d G-buffer on z = 0, %d quad lights, %s, plain LTC-RIS M=%d, %d spp"
                % (a.width, a.height, a.lights, "%s occluder triangles" % count_name(a.triangles) if a.triangles
                   else "unshadowed", a.candidates, a.spp))
    return ("shadowed single frame: %dx%d fBm heightfield, %d polygon lights (3-8 vertices), %s occluder "
            "triangles (SAH BVH), plain LTC-RIS M=%d, %d spp" % (a.width, a.height, a.lights,
                                                                count_name(a.triangles), a.candidates, a.spp))
METRIC = "Gsamples/s (plain LTC-RIS, shadowed 1080p frame, 1024 lights, M=32, 4 spp)"


def metric_name(a):
    """The headline metric's name for its own workload (1080p heightfield,
    1024 lights, 200k occluders, M = 32, 4 spp), else one naming the workload."""
    headline = (a.scene == "heightfield" and (a.width, a.height, a.lights, a.triangles, a.candidates, a.spp)
                == (1920, 1080, 1024, 200_000, 32, 4))
    return METRIC if headline else "Gsamples/s (%s)" % workload_name(a)


L2_BYTES = 129 * 1024 * 1024


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--scene", choices=["heightfield", "plane"], default="heightfield",
                   help="plane: the plane-of-quads form (G-buffer on z = 0, quad lights)")
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--lights", type=int, default=1024)
    p.add_argument("--triangles", type=int, default=200_000)
    p.add_argument("--candidates", type=int, default=32)
    p.add_argument("--spp", type=int, default=4)
    p.add_argument("--numerics", choices=["exact", "fast"], default="exact")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--clocks-csv", default=None, help="keep the raw nvidia-smi clock samples in this file")
    p.add_argument("--workload", choices=["throughput", "equal-mse", "batch"], default="throughput",
                   help="equal-mse: device time to equal MSE, learned cluster proposal vs plain RIS; batch: 16 "
                        "plane-of-quads scenes of mixed sizes in one autotuned, graph-captured batched launch")
    p.add_argument("--batch-scenes", type=int, default=16)
    p.add_argument("--batch-candidates", type=int, default=8)
    p.add_argument("--clusters", type=int, default=256)
    p.add_argument("--train-frames", type=int, default=64)
    p.add_argument("--reference-spp", type=int, default=4096)
    p.add_argument("--shadowed-target", type=float, default=0.5,
                   help="weight of the shadowed (visibility) part of the learned proposal's training target")
    p.add_argument("--learning-rate", type=float, default=5e-3,
                   help="equal-mse: the learned proposal's Adam step (measured: 1e-3 trains too slowly in 64 frames, "
                        "5e-3 and 1e-2 equally well)")
    p.add_argument("--train-stride", type=int, default=16, help="equal-mse: every n-th pixel trains the model")
    p.add_argument("--train-on-cuda-cores", action="store_true",
                   help="equal-mse: train with the FP32 CUDA-core kernel instead of the tensor cores")
    p.add_argument("--uniform-fraction", type=float, default=0.05,
                   help="equal-mse: weight of uniform light choice in the proposals' defensive mixture (measured on "
                        "960x540: 0.05 gives a lower MSE than 0.1 for both proposals)")
    p.add_argument("--sweep-candidates", default="",
                   help="equal-mse: also measure every method at these candidate counts (comma-separated); plain "
                        "RIS at --candidates stays the MSE level to reach")
    return p.parse_args()


def make_workload(a, seed=0):
    from risltc_gb300 import scenes
    if a.scene == "plane":
        return scenes.plane_of_quads(a.width, a.height, a.lights, seed=seed, triangles=a.triangles)
    return scenes.heightfield(a.width, a.height, light_count=a.lights, triangle_count=a.triangles, seed=seed,
                              vertex_counts=(3, 8))


# ----------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi clock and throttle-reason samples (every 50 ms, started
    before the warm-up so that it is running when the timed region begins);
    stop() keeps the samples taken between mark_start() and mark_stop()."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0, path=None):
        """path: where the raw samples go (kept); default a temporary file,
        removed by stop()."""
        self.proc = None
        self.t0 = self.t1 = None
        self.keep = path is not None
        if path is None:
            fd, path = tempfile.mkstemp(prefix="risltc_clocks_", suffix=".csv")
            os.close(fd)
        self.path = path
        try:
            os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device_index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def mark_start(self):
        self.t0 = time.time()

    def mark_stop(self):
        self.t1 = time.time()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.f.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 10 or not parts[2].replace(".", "").isdigit():
                    continue
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                except ValueError:
                    ts = None
                rows.append((ts, parts[1:]))
        if not self.keep:
            os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        window = [r for ts, r in rows if ts is not None and self.t0 is not None and self.t0 <= ts <= self.t1]
        note = "samples inside the timed region"
        if not window:
            window = [r for _, r in rows]
            note = "no sample fell inside the timed region: all samples of the run"
        sm = [float(r[1]) for r in window]
        smax = max(float(r[2]) for r in window)
        power = [float(r[3]) for r in window if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in window for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": reasons, "samples": len(window),
                "power_w_max": max(power) if power else None, "note": note}


def measured_traffic(kernel, samples_per_step):
    """DRAM bytes (read + write) per launch of `kernel` for this step, from the
    ncu capture summarised in profiles/traffic.json, scaled from the captured
    launch's pixel-samples to this step's (the traffic grows with them)."""
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            t = json.load(f)[kernel]
        return t["dram_bytes"] * samples_per_step / t["pixel_samples"], t["source"]
    except (OSError, ValueError, KeyError):
        return None, None


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# --------------------------------------------------------------- CPU leg --
def _pixel_subset(hs, count, seed):
    """A 1-row G-buffer of `count` pixels drawn uniformly from the frame's
    covered pixels (an unbiased sample of the per-pixel cost)."""
    valid = np.flatnonzero(hs.primitive == 0) if hs.primitive is not None else np.arange(hs.pixels)
    pick = np.sort(np.random.default_rng(seed).choice(valid, size=min(count, valid.size), replace=False))
    return np.ascontiguousarray(hs.gbuffer[:, pick]), pick.size


def cpu_sample(hs, a, seconds_target, threads=0, seed=1, count_ops=True, repeats=1):
    """Times the FP32 oracle (the reference's routines restated in C99,
    OpenMP over rows) on pixels drawn uniformly from the same frame, and
    counts the algorithmic FP32 operations per pixel-sample with the
    op-counting build of the same oracle."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from risltc_gb300 import api
    nodes, tris, _, _ = api.build_bvh(hs.triangles)
    osc = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants, tris, nodes)
    st = oracle.make_settings(candidates=a.candidates)
    rn = api.noise_constants(0)[0]
    nthreads = threads or oracle.max_threads()
    # Rows of 256 pixels so OpenMP has rows to balance.
    probe, n = _pixel_subset(hs, 256 * nthreads, seed)
    _, _, t = oracle.render(osc, st, probe, 256, n // 256, rn, threads=nthreads, reservoirs=False)
    want = int(256 * (n // 256) * seconds_target / max(t, 1e-3))
    want = max(256, min(want // 256 * 256, hs.pixels // 256 * 256))
    sample, n = _pixel_subset(hs, want, seed + 1)
    rows = n // 256
    times = []
    for _ in range(repeats):
        _, _, t = oracle.render(osc, st, sample[:, :rows * 256], 256, rows, rn, threads=nthreads, reservoirs=False)
        times.append(t)
    out = {"samples": rows * 256, "seconds": statistics.median(times), "times": times, "threads": nthreads}
    if count_ops:
        # Counted with M and with one candidate: the difference is the
        # candidate phase, the rest the final PSA/MIS shading.
        ops_g, m = _pixel_subset(hs, 1024, seed + 2)
        # Counted once more without occluders: the difference is the
        # shadow rays' BVH traversal.
        ops = oracle.opcount(osc, st, ops_g, m, 1, rn, (0, 1))
        one = oracle.opcount(osc, oracle.make_settings(candidates=1), ops_g, m, 1, rn, (0, 1))
        unshadowed = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants)
        lit = oracle.opcount(unshadowed, st, ops_g, m, 1, rn, (0, 1))
        per_candidate = (ops["flops"] - one["flops"]) / m / max(a.candidates - 1, 1)
        out["flops_per_sample"] = ops["flops"] / m
        out["candidate_flops_per_sample"] = per_candidate * a.candidates
        out["shade_flops_per_sample"] = lit["flops"] / m - per_candidate * a.candidates
        out["trace_flops_per_sample"] = (ops["flops"] - lit["flops"]) / m
        # Traversal bytes of the same queries on the identical BVH: 32 bytes
        # per box tested (the device reads a child pair's two boxes, 64 bytes,
        # per inner node) and 48 per triangle tested.
        out["trace_bytes_per_sample"] = (32.0 * ops["boxes"] + 48.0 * ops["triangles"]) / m
        out["ops"] = {k: v for k, v in ops.items() if k != "rgb"}
    return out


def run_reference(a, rank, world):
    """--impl reference: the oracle port of the reference's shading routines
    (FP32, C99, OpenMP over all host threads) on a bounded band per step."""
    if rank != 0:
        return
    hs = make_workload(a)
    # Warm-up steps are folded into the probe; each timed step re-renders the
    # same uniformly drawn pixel sample.
    info = cpu_sample(hs, a, seconds_target=min(a.cpu_seconds, 8.0), count_ops=False, repeats=a.steps)
    value = info["samples"] / info["seconds"] / 1e9
    line = {
        "impl": "reference", "metric": metric_name(a), "value": value, "unit": "Gsamples/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000.0 * info["seconds"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(a), "sample": "%d pixels drawn uniformly from the frame, 1 spp" % (
            info["samples"])},
        "cpu_baseline": {"value": value, "unit": "Gsamples/s", "cores": info["threads"], "kind": "port",
                         "sample": "%d pixel-samples drawn uniformly from the frame per step, FP32 oracle "
                                   "(C99, OpenMP)" % info["samples"]},
        "e2e": {"value": value, "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU leg --
def run_ours(a, rank, world, local_rank):
    import torch
    import risltc_gb300 as rl
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    hs = make_workload(a, seed=0)
    P = hs.pixels
    samples_per_step = int((hs.primitive == 0).sum() if hs.primitive is not None else P) * a.spp
    ctx = rl.Context(local_rank)
    scene = rl.Scene.from_host_scene(ctx, hs)
    s = rl.settings(candidates=a.candidates, numerics=a.numerics)
    g = torch.from_numpy(hs.gbuffer).cuda()
    prim = torch.from_numpy(hs.primitive.view(np.int32)).cuda() if hs.primitive is not None else None
    out = torch.empty((P, 3), dtype=torch.float32, device="cuda")
    # Each rank shades different frames (its own noise seeds).
    seed = rank * 1_000_000
    clocks = ClockSampler(local_rank, a.clocks_csv) if rank == 0 else None
    for _ in range(a.warmup):
        seed = rl.shade(ctx, scene, g, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, out_rgb=out,
                        primitive=prim)
    ctx.check()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.profile(True)  # per-kernel CUDA events on the same stream
    if clocks:
        clocks.mark_start()
    # Inputs smaller than L2: flush it (write a 256 MB buffer) before every
    # timed step, outside that step's events.
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if hs.gbuffer.nbytes <= L2_BYTES else None
    step_events = []
    start.record(stream)
    for _ in range(a.steps):
        if flush is not None:
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        seed = rl.shade(ctx, scene, g, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, out_rgb=out,
                        primitive=prim)
        if flush is not None:
            e1.record(stream)
            step_events.append((e0, e1))
    stop.record(stream)
    torch.cuda.synchronize()
    if clocks:
        clocks.mark_stop()
    if dist:
        dist.barrier()
    clock_info = clocks.stop() if clocks else None
    prof = ctx.profile(False)
    ctx.check()
    # The same step with the other numerics mode, for reference (exact is
    # bit-identical to the oracle; fast approximates the candidate loop).
    other = "fast" if a.numerics == "exact" else "exact"
    exact_s = rl.settings(candidates=a.candidates, numerics=other)
    rl.shade(ctx, scene, g, hs.width, hs.height, exact_s, noise_seed=seed, frames=a.spp, out_rgb=out, primitive=prim)
    torch.cuda.synchronize()
    other_events = []
    for _ in range(a.steps):
        if flush is not None:
            flush.fill_(1)
        o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        o0.record(stream)
        seed = rl.shade(ctx, scene, g, hs.width, hs.height, exact_s, noise_seed=seed, frames=a.spp, out_rgb=out,
                        primitive=prim)
        o1.record(stream)
        other_events.append((o0, o1))
    torch.cuda.synchronize()
    other_value = samples_per_step * a.steps / (sum(o0.elapsed_time(o1) for o0, o1 in other_events) / 1000.0) / 1e9
    elapsed = start.elapsed_time(stop) / 1000.0
    if step_events:
        elapsed = sum(e0.elapsed_time(e1) for e0, e1 in step_events) / 1000.0
    t = torch.tensor([elapsed], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    elapsed = float(t.item())
    value = samples_per_step * world * a.steps / elapsed / 1e9
    ms_per_step = 1000.0 * elapsed / a.steps
    result = {"value": value, "ms_per_step": ms_per_step}

    # End to end through the host entry point: pinned G-buffer in, RGB out.
    e2e = None
    if not a.no_e2e:
        hg = torch.from_numpy(hs.gbuffer).pin_memory()
        hp = torch.from_numpy(hs.primitive.view(np.int32)).pin_memory() if hs.primitive is not None else None
        ho = torch.empty((P, 3), dtype=torch.float32).pin_memory()
        hgn, hon = hg.numpy(), ho.numpy()
        hpn = hp.numpy().view(np.uint32) if hp is not None else None
        for _ in range(max(1, a.warmup // 2)):
            rl.shade_host(ctx, scene, hgn, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, primitive=hpn,
                          out=hon)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            rl.shade_host(ctx, scene, hgn, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, primitive=hpn,
                          out=hon)
            seed += a.spp
        te = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device="cuda")
        if dist:
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
        e2e = {"value": samples_per_step * world * a.steps / float(te.item()) / 1e9, "unit": "Gsamples/s",
               "h2d_bytes_per_step": int(hs.gbuffer.nbytes + (hs.primitive.nbytes if hs.primitive is not None else 0)),
               "d2h_bytes_per_step": int(P * 3 * 4)}
    scene.close()
    ctx.close()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks = measured_peaks()
    props = torch.cuda.get_device_properties(local_rank)
    sms = props.multi_processor_count
    sm_max = peaks.get("sm_max_mhz") or (clock_info or {}).get("sm_max_mhz") or 2070.0
    fp32_peak = 2.0 * 128 * sms * sm_max * 1e6 / 1e12  # TFLOP/s, 128 FP32 lanes per SM
    cpu = None
    flops_per_sample = None
    info = {}
    if not a.no_cpu_baseline:
        info = cpu_sample(hs, a, a.cpu_seconds)
        flops_per_sample = info["flops_per_sample"]
        cpu = {"value": info["samples"] / info["seconds"] / 1e9, "unit": "Gsamples/s", "cores": info["threads"],
               "kind": "port", "sample": "%d pixel-samples drawn uniformly from the same frame at 1 spp, FP32 "
                                         "oracle (C99, OpenMP over rows of 256)" % info["samples"]}
    roofline = None
    calls = max(prof["calls"], 1)
    # One launch of each kernel per step (all spp frames in one call).  The
    # resolve kernel's few operations are counted with the sample kernel.
    kernels = {"ris_candidates_binned_kernel": {"ms_per_launch": prof["candidates"] / calls},
               "ris_sample_kernel": {"ms_per_launch": prof["shade"] / calls},
               "shadow_trace_kernel": {"ms_per_launch": prof["shadow_trace"] / calls},
               "ris_resolve_kernel": {"ms_per_launch": prof["resolve"] / calls}}
    if flops_per_sample:
        kernels["ris_candidates_binned_kernel"]["flops_per_sample"] = info["candidate_flops_per_sample"]
        kernels["ris_sample_kernel"]["flops_per_sample"] = info["shade_flops_per_sample"]
        kernels["shadow_trace_kernel"]["flops_per_sample"] = info["trace_flops_per_sample"]
        tk = kernels["shadow_trace_kernel"]
        tk["bytes_per_sample"] = info["trace_bytes_per_sample"]
        tk["achieved_gbs"] = (tk["bytes_per_sample"] * samples_per_step / (tk["ms_per_launch"] / 1e3) / 1e9
                              if tk["ms_per_launch"] > 0 else 0.0)
        if peaks.get("hbm_gbs"):
            # The BVH (about 14 MB) stays in L2/L1, so this is the node and
            # triangle traffic the traversal moves, against HBM copy bandwidth
            # for scale (ray sort included in the timed phase).
            tk["gbs_frac_of_hbm"] = tk["achieved_gbs"] / peaks["hbm_gbs"]
        kernels["ris_resolve_kernel"]["flops_per_sample"] = 0.0
        for k in kernels.values():
            k["achieved_tflops"] = (k["flops_per_sample"] * samples_per_step / (k["ms_per_launch"] / 1e3) / 1e12
                                    if k["ms_per_launch"] > 0 else 0.0)
            k["frac"] = k["achieved_tflops"] / fp32_peak
        dominant = max(kernels, key=lambda k: kernels[k]["ms_per_launch"])
        d = kernels[dominant]
        traffic, traffic_source = measured_traffic(dominant, samples_per_step)
        roofline = {"bound": "fp32", "achieved": d["achieved_tflops"], "peak": fp32_peak, "unit": "TFLOP/s",
                    "frac": d["frac"], "traffic": traffic, "traffic_source": traffic_source, "kernel": dominant,
                    "flops_per_sample": d["flops_per_sample"],
                    "whole_step_frac": flops_per_sample * samples_per_step / (elapsed / a.steps) / 1e12 / fp32_peak,
                    "peak_source": "derived: 2 x 128 FP32 lanes x %d SMs x %.0f MHz (max SM clock of "
                                   "MEASURED_PEAKS.json); no measured FP32 peak exists" % (sms, sm_max)}
    line = {
        "metric": metric_name(a), "value": result["value"], "unit": "Gsamples/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": result["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(a), "width": hs.width, "height": hs.height, "lights": hs.light_count,
                   "triangles": int(hs.triangles.shape[0]), "candidates": a.candidates, "spp": a.spp,
                   "numerics": a.numerics, "samples_per_step": samples_per_step,
                   "l2": ("inputs larger than L2 (G-buffer %.0f MB > 129 MB)" if hs.gbuffer.nbytes > L2_BYTES else
                          "inputs smaller than L2 (G-buffer %.0f MB < 129 MB): L2 flushed (256 MB written) before "
                          "every timed step, outside its events") % (hs.gbuffer.nbytes / 1e6),
                   "parallelism": "one frame per GPU" if world > 1 else "single GPU"},
        "gpu_launches": 4 * a.steps,
        "kernels": kernels,
        "other_numerics": {"numerics": other, "value": other_value, "unit": "Gsamples/s"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clock_info,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_equal_mse(a):
    """Device time to equal MSE, learned cluster proposal vs plain RIS.

    Heightfield frame with a.lights lights k-means-grouped into a.clusters
    clusters and a.triangles occluders.  Reference: a.reference_spp spp of
    plain RIS accumulated in FP64 on the GPU.  The learned proposal's model
    trains online for a.train_frames frames first (1 spp each, every 16th
    pixel); then each method renders a.spp spp four times with fresh noise
    and its MSE against the reference is measured, with its device time per
    frame (CUDA events over a.steps calls of a.spp frames each, the same
    calls that the MSE is measured on; training off).  MSE falls as 1 / spp for these
    unbiased estimators, so the time to reach plain RIS's a.spp-spp MSE is
    ms_per_frame * spp * MSE(method) / MSE(plain)."""
    import torch
    import risltc_gb300 as rl
    from risltc_gb300 import scenes
    hs0 = make_workload(a, seed=0)
    hs, offsets = scenes.cluster_lights(hs0, a.clusters, seed=1)
    ctx = rl.Context(0)
    scene = rl.Scene.from_host_scene(ctx, hs)
    scene.set_clusters(offsets)
    model = rl.Model(ctx, a.clusters, seed=2)
    model.set_input_transform((0.0, 0.0, 1.0), 6.0)
    scene.set_model(model)
    P = hs.pixels
    covered = torch.from_numpy(hs.primitive == 0).cuda() if hs.primitive is not None else None
    g = torch.from_numpy(hs.gbuffer).cuda()
    prim = torch.from_numpy(hs.primitive.view(np.int32)).cuda()
    plain = rl.settings(candidates=a.candidates)
    clusters = rl.settings(candidates=a.candidates, proposal="clusters", proposal_uniform_fraction=a.uniform_fraction)
    learned = rl.settings(candidates=a.candidates, proposal="learned", proposal_uniform_fraction=a.uniform_fraction)
    # Reference: FP64 running sums of plain RIS.
    acc = torch.zeros((P, 3), dtype=torch.float64, device="cuda")
    seed = 10_000_000
    for _ in range(a.reference_spp // 16):
        seed = rl.shade(ctx, scene, g, hs.width, hs.height, plain, noise_seed=seed, frames=16, accum=acc,
                        primitive=prim)
    reference = acc / (16 * (a.reference_spp // 16))
    ctx.check()
    # Online training of the model (1 spp per call, its own candidates).
    model.set_training(True, learning_rate=a.learning_rate, pixel_stride=a.train_stride)
    model.set_training_flags(cuda_cores=a.train_on_cuda_cores)
    model.set_target_mix(a.shadowed_target)
    out = torch.empty((P, 3), dtype=torch.float32, device="cuda")
    seed = 20_000_000
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(a.train_frames):
        seed = rl.shade(ctx, scene, g, hs.width, hs.height, learned, noise_seed=seed, frames=1, out_rgb=out,
                        primitive=prim)
    t1.record()
    torch.cuda.synchronize()
    train_ms = t0.elapsed_time(t1) / max(a.train_frames, 1)
    model.set_training(False)
    results = {}
    runs = [("plain", plain), ("clusters", clusters), ("learned", learned)]
    for m in [int(x) for x in a.sweep_candidates.split(",") if x.strip()]:
        if m != a.candidates:
            runs += [("%s_m%d" % (name, m), rl.copy_settings(st, candidate_count=m)) for name, st in runs[:3]]
    for name, s in runs:
        mses = []
        for rep in range(4):
            rl.shade(ctx, scene, g, hs.width, hs.height, s, noise_seed=30_000_000 + 1000 * rep, frames=a.spp,
                     out_rgb=out, primitive=prim)
            d = (out.double() - reference) ** 2
            if covered is not None:
                d = d[covered]
            mses.append(float(d.mean()))
        # Device time of the same a.spp-frame calls whose MSE was measured
        # (per-call work, such as the logits and the cluster distributions,
        # is shared by the call's frames).
        for _ in range(a.warmup):
            rl.shade(ctx, scene, g, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, out_rgb=out,
                     primitive=prim)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(a.steps):
            rl.shade(ctx, scene, g, hs.width, hs.height, s, noise_seed=40_000_000 + a.spp * i, frames=a.spp,
                     out_rgb=out, primitive=prim)
        e1.record()
        torch.cuda.synchronize()
        results[name] = {"mse_at_spp": statistics.mean(mses), "ms_per_frame": e0.elapsed_time(e1) / (a.spp * a.steps),
                         "candidates": int(s.candidate_count)}
    ctx.check()
    base = results["plain"]
    for r in results.values():
        r["ms_to_plain_mse"] = r["ms_per_frame"] * a.spp * r["mse_at_spp"] / base["mse_at_spp"]
    # Each method at its best candidate count (of those measured).
    best = {}
    for method in ("plain", "clusters", "learned"):
        keys = [k for k in results if k == method or k.startswith(method + "_m")]
        k = min(keys, key=lambda k: results[k]["ms_to_plain_mse"])
        best[method] = {"run": k, "candidates": results[k]["candidates"],
                        "ms_to_plain_mse": results[k]["ms_to_plain_mse"]}
    line = {
        "metric": "ms/frame to equal MSE, learned-proposal vs plain RIS (%dx%d, %d lights); Gsamples/s"
                  % (hs.width, hs.height, hs.light_count),
        "value": best["learned"]["ms_to_plain_mse"], "unit": "ms", "higher_is_better": False,
        "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "dtype": "f32 (MLP bf16/fp32)", "data": "synthetic",
        "config": {"workload": "equal MSE: %dx%d fBm heightfield, %d polygon lights (3-8 vertices) in %d k-means "
                               "clusters, %dk occluder triangles, M=%d, MSE at %d spp against a %d-spp FP64 plain-RIS "
                               "reference" % (hs.width, hs.height, hs.light_count, a.clusters, a.triangles // 1000,
                                              a.candidates, a.spp, a.reference_spp),
                   "train_frames": a.train_frames, "train_ms_per_frame": train_ms, "learning_rate": a.learning_rate,
                   "train_stride": a.train_stride, "uniform_fraction": a.uniform_fraction,
                   "training": "cuda cores fp32" if a.train_on_cuda_cores or a.clusters > 256 else "tensor cores bf16",
                   "shadowed_target": a.shadowed_target},
        "plain_ms_to_equal_mse": base["ms_to_plain_mse"],
        "speedup_vs_plain": base["ms_to_plain_mse"] / results["learned"]["ms_to_plain_mse"],
        "best_candidate_count": best,
        "speedup_best_vs_plain": base["ms_to_plain_mse"] / best["learned"]["ms_to_plain_mse"],
        "speedup_best_vs_best_plain": best["plain"]["ms_to_plain_mse"] / best["learned"]["ms_to_plain_mse"],
        "methods": results,
        "gsamples_per_s": {k: hs.pixels / (v["ms_per_frame"] / 1e3) / 1e9 for k, v in results.items()},
    }
    print(json.dumps(line), flush=True)
    scene.close()
    model.close()
    ctx.close()


def batch_workload(count, seed=3):
    """Scenes of the plane-of-quads form (G-buffer on z = 0, quads above it)
    with log-uniform resolutions between 256x256 and 1920x1080, light counts
    16..8192 and occluder counts 10k..500k."""
    from risltc_gb300 import scenes
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        t = rng.uniform(0.0, 1.0)
        w, h = int(round(256 * (1920 / 256) ** t)), int(round(256 * (1080 / 256) ** t))
        lights = int(np.exp(rng.uniform(np.log(16), np.log(8192))))
        tris = int(np.exp(rng.uniform(np.log(10_000), np.log(500_000))))
        out.append(scenes.plane_of_quads(w, h, lights, seed=seed * 1000 + i, triangles=tris))
    return out


def run_batch(a):
    """Batched launch: a.batch_scenes scenes shaded by one risltc_shade_batch
    call per step, captured once into a CUDA graph and replayed, with the
    candidate kernel's tile shape picked by risltc_autotune_batch."""
    import torch
    import risltc_gb300 as rl
    hss = batch_workload(a.batch_scenes)
    stream = torch.cuda.Stream()
    ctx = rl.Context(0, stream=stream.cuda_stream)
    scenes_ = [rl.Scene.from_host_scene(ctx, hs) for hs in hss]
    s = rl.settings(candidates=a.batch_candidates, numerics=a.numerics)
    samples_per_step = sum(hs.pixels for hs in hss)
    items = []
    with torch.cuda.stream(stream):
        for k, (hs, sc) in enumerate(zip(hss, scenes_)):
            items.append(dict(scene=sc, gbuffer=torch.from_numpy(hs.gbuffer).cuda(), width=hs.width,
                              height=hs.height, settings=s, noise_seed=1000 * k, frames=1,
                              out_rgb=torch.empty((hs.pixels, 3), dtype=torch.float32, device="cuda")))
        rl.shade_batch(ctx, items)  # sizes the scratch and creates the streams
    torch.cuda.synchronize()
    tile, tile_ms = rl.autotune_batch(ctx, items, repeats=3)
    with torch.cuda.stream(stream):
        for _ in range(a.warmup):
            rl.shade_batch(ctx, items)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        rl.shade_batch(ctx, items)
    # Replays go to the current stream: the context's, where the events are.
    with torch.cuda.stream(stream):
        for _ in range(a.warmup):
            graph.replay()
    torch.cuda.synchronize()
    ctx.check()
    clocks = ClockSampler(0, a.clocks_csv)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.mark_start()
    with torch.cuda.stream(stream):
        start.record(stream)
        for _ in range(a.steps):
            graph.replay()
        stop.record(stream)
    torch.cuda.synchronize()
    clocks.mark_stop()
    clock_info = clocks.stop()
    ctx.check()
    elapsed = start.elapsed_time(stop) / 1000.0
    value = samples_per_step * a.steps / elapsed / 1e9
    # End to end through the public API: every item's G-buffer copied in from
    # pinned host memory, the batch call, every image copied back.
    e2e = None
    if not a.no_e2e:
        host_g = [torch.from_numpy(hs.gbuffer).pin_memory() for hs in hss]
        host_o = [torch.empty((hs.pixels, 3), dtype=torch.float32).pin_memory() for hs in hss]

        def e2e_step():
            with torch.cuda.stream(stream):
                for it, hg in zip(items, host_g):
                    it["gbuffer"].copy_(hg, non_blocking=True)
                rl.shade_batch(ctx, items)
                for it, ho in zip(items, host_o):
                    ho.copy_(it["out_rgb"], non_blocking=True)
            stream.synchronize()
        e2e_step()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            e2e_step()
        te = time.perf_counter() - t0
        ctx.check()
        e2e = {"value": samples_per_step * a.steps / te / 1e9, "unit": "Gsamples/s",
               "h2d_bytes_per_step": int(sum(hs.gbuffer.nbytes for hs in hss)),
               "d2h_bytes_per_step": int(sum(hs.pixels * 12 for hs in hss))}
    cpu = None
    if not a.no_cpu_baseline:
        samples = seconds = 0.0
        threads = 1
        for hs in hss:
            sub = argparse.Namespace(**vars(a))
            sub.candidates = a.batch_candidates
            info = cpu_sample(hs, sub, a.cpu_seconds / len(hss), count_ops=False)
            samples += info["samples"]
            seconds += info["seconds"]
            threads = info["threads"]
        cpu = {"value": samples / seconds / 1e9, "unit": "Gsamples/s", "cores": threads, "kind": "port",
               "sample": "%d pixel-samples drawn uniformly from the %d scenes (about %.1f s of CPU work each), "
                         "FP32 oracle (C99, OpenMP over rows of 256)" % (samples, len(hss),
                                                                        a.cpu_seconds / len(hss))}
    for sc in scenes_:
        sc.close()
    ctx.close()
    line = {
        "metric": "Gsamples/s (batched graph launch: %d plane-of-quads scenes, 256^2..1080p, 16..8192 lights, "
                  "10k..500k occluders, M=%d, 1 spp)" % (len(hss), a.batch_candidates),
        "value": value, "unit": "Gsamples/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1000.0 * elapsed / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batch of %d scenes in one CUDA-graph replay of risltc_shade_batch (8 streams)"
                               % len(hss),
                   "scenes": [{"width": hs.width, "height": hs.height, "lights": hs.light_count,
                               "triangles": int(hs.triangles.shape[0])} for hs in hss],
                   "candidates": a.batch_candidates, "numerics": a.numerics, "samples_per_step": samples_per_step,
                   "tile": tile, "autotune_ms_per_batch": tile_ms,
                   "l2": "inputs larger than L2 (G-buffers %.0f MB > 129 MB)"
                         % (sum(hs.gbuffer.nbytes for hs in hss) / 1e6)},
        "gpu_launches": 6 * len(hss) * a.steps,
        "roofline": None,
        "roofline_note": "kernels of 8 streams overlap inside the batch; the per-kernel roofline is reported by "
                         "the single-frame throughput workload",
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clock_info,
    }
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if a.workload == "equal-mse":
        if rank == 0 and a.impl == "ours":
            run_equal_mse(a)
        return
    if a.workload == "batch":
        if rank == 0 and a.impl == "ours":
            run_batch(a)
        return
    if a.impl == "reference":
        run_reference(a, rank, world)
    else:
        run_ours(a, rank, world, local_rank)


if __name__ == "__main__":
    main()
