"""Benchmark of the shading path on the workload of the headline metric.

Default workload (the many-lights frame): a 1920x1080 G-buffer of a seeded
fBm heightfield, 16,384 convex polygon lights with 3..8 vertices (areas
log-uniform [0.01, 1]) k-means-grouped into 256 clusters, 1M random occluder
triangles (edge 0.05..0.5) in [-6, 6]^2 x [0, 2] behind a SAH BVH.  One step
shades one 4-spp call of plain LTC-RIS with M = 32 candidates (all frames
in one launch of each kernel).  The line reports:

  value        pixel-samples per second of plain RIS, inputs resident in HBM
               (one sample = M candidates + the PSA/MIS shade with its
               shadow rays);
  e2e          the same through risltc_shade_host (host buffers, copies
               inside the timed region);
  equal_mse    device time to plain RIS's MSE, learned cluster proposal
               (trained online for 64 frames on the tensor cores) against
               plain RIS and the heuristic cluster proposal;
  parity       the GPU's frame against the oracle on the CPU-baseline
               sample (bit-exact pixels expected);
  rates        candidates per second and shadow rays per second;
  roofline, cpu_baseline, clocks, gpu_launches, kernels, config2 (the
               1024-light, 200k-occluder frame's throughput).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                  [--workload headline|throughput|equal-mse|batch]

Prints one JSON line (rank 0).  N > 1 runs one process per GPU (torchrun),
each shading its own frames (weak scaling, no data-path collective).
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

HEADLINE_METRIC = "ms/frame to equal MSE, learned-proposal vs plain RIS (1080p, 16K lights); Gsamples/s"
# Workload sizes per --workload where the command line leaves them open.
DEFAULTS = {
    "headline": dict(width=1920, height=1080, lights=16384, triangles=1_000_000, clusters=256),
    "throughput": dict(width=1920, height=1080, lights=1024, triangles=200_000, clusters=0),
    "equal-mse": dict(width=1920, height=1080, lights=16384, triangles=1_000_000, clusters=256),
    "batch": dict(width=1920, height=1080, lights=1024, triangles=200_000, clusters=0),
}


def count_name(n):
    """200000 -> '200k'; counts that are not whole thousands as they are."""
    return "%dk" % (n // 1000) if n >= 1000 and n % 1000 == 0 else str(n)


def workload_name(a):
    if a.scene == "plane":
        return ("plane of quads: %dx%d G-buffer on z = 0, %d quad lights, %s, plain LTC-RIS M=%d, %d spp"
                % (a.width, a.height, a.lights, "%s occluder triangles" % count_name(a.triangles) if a.triangles
                   else "unshadowed", a.candidates, a.spp))
    clusters = " in %d k-means clusters" % a.clusters if a.clusters else ""
    return ("%s: %dx%d fBm heightfield, %d polygon lights (3-8 vertices)%s, %s occluder triangles (SAH BVH), "
            "plain LTC-RIS M=%d, %d spp" % ("many-lights frame" if a.clusters else "shadowed single frame", a.width,
                                            a.height, a.lights, clusters, count_name(a.triangles), a.candidates,
                                            a.spp))


def is_headline(a):
    return (a.scene == "heightfield" and (a.width, a.height, a.lights, a.triangles, a.clusters, a.candidates, a.spp)
            == (1920, 1080, 16384, 1_000_000, 256, 32, 4))


def metric_name(a):
    """The headline metric's name for its own workload, else one naming the
    workload."""
    return HEADLINE_METRIC if is_headline(a) else "Gsamples/s (%s)" % workload_name(a)


L2_BYTES = 129 * 1024 * 1024


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["headline", "throughput", "equal-mse", "batch"], default="headline",
                   help="headline: the many-lights frame's plain-RIS throughput with its equal-MSE comparison and "
                        "the 1024-light frame's throughput; throughput: one frame's throughput alone; equal-mse: "
                        "the equal-MSE comparison alone; batch: 16 plane-of-quads scenes of mixed sizes in one "
                        "autotuned, graph-captured batched launch")
    p.add_argument("--scene", choices=["heightfield", "plane"], default="heightfield",
                   help="plane: the plane-of-quads form (G-buffer on z = 0, quad lights)")
    p.add_argument("--width", type=int, default=None)
    p.add_argument("--height", type=int, default=None)
    p.add_argument("--lights", type=int, default=None)
    p.add_argument("--triangles", type=int, default=None)
    p.add_argument("--clusters", type=int, default=None,
                   help="k-means light clusters (0: lights in generation order, no cluster proposal)")
    p.add_argument("--candidates", type=int, default=32)
    p.add_argument("--spp", type=int, default=4)
    p.add_argument("--numerics", choices=["exact", "fast"], default="exact")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the baseline sample")
    p.add_argument("--parity-pixels", type=int, default=4096,
                   help="pixels of the frame checked against the oracle (at least this many; the CPU-baseline "
                        "sample when larger)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-equal-mse", action="store_true", help="headline: leave out the equal-MSE comparison")
    p.add_argument("--no-config2", action="store_true", help="headline: leave out the 1024-light frame")
    p.add_argument("--clocks-csv", default=None, help="keep the raw nvidia-smi clock samples in this file")
    p.add_argument("--batch-scenes", type=int, default=16)
    p.add_argument("--batch-candidates", type=int, default=8)
    p.add_argument("--train-frames", type=int, default=64)
    p.add_argument("--reference-spp", type=int, default=4096)
    p.add_argument("--mse-spp", type=int, default=16, help="equal-mse: frames per call whose MSE is measured")
    p.add_argument("--mse-steps", type=int, default=8, help="equal-mse: timed calls per method")
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
    p.add_argument("--sweep-candidates", default="8,16",
                   help="equal-mse: also measure every method at these candidate counts (comma-separated); plain "
                        "RIS at --candidates stays the MSE level to reach")
    a = p.parse_args(argv)
    for k, v in DEFAULTS[a.workload].items():
        if getattr(a, k) is None:
            setattr(a, k, v)
    return a


def make_workload(a, seed=0):
    """The host scene of a's workload; with a.clusters > 0 its lights are
    listed cluster by cluster.  Returns (scene, cluster offsets or None)."""
    from risltc_gb300 import scenes
    if a.scene == "plane":
        return scenes.plane_of_quads(a.width, a.height, a.lights, seed=seed, triangles=a.triangles), None
    hs = scenes.heightfield(a.width, a.height, light_count=a.lights, triangle_count=a.triangles, seed=seed,
                            vertex_counts=(3, 8))
    if a.clusters:
        return scenes.cluster_lights(hs, a.clusters, seed=1)
    return hs, None


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


def measured_traffic(kernel, workload, samples_per_step):
    """DRAM bytes (read + write) per launch of `kernel` on `workload` (a key
    of profiles/traffic.json, from an ncu capture), scaled from the captured
    launch's pixel-samples to this step's (the traffic grows with them)."""
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            t = json.load(f)[workload][kernel]
        return t["dram_bytes"] * samples_per_step / t["pixel_samples"], t["source"]
    except (OSError, ValueError, KeyError):
        return None, None


def traffic_key(a):
    if is_headline(a):
        return "many_lights_1080p"
    if (a.scene, a.width, a.height, a.lights, a.triangles, a.candidates) == ("heightfield", 1920, 1080, 1024,
                                                                             200_000, 32):
        return "shadowed_1080p_1024_lights"
    return None


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# --------------------------------------------------------------- CPU leg --
def _covered(hs):
    return np.flatnonzero(hs.primitive == 0) if hs.primitive is not None else np.arange(hs.pixels)


def _pixel_sample(hs, count, seed):
    """`count` pixel indices drawn uniformly without replacement from the
    frame's covered pixels, ascending."""
    valid = _covered(hs)
    if count >= valid.size:
        return valid.astype(np.uint32)
    return np.sort(np.random.default_rng(seed).choice(valid, size=count, replace=False)).astype(np.uint32)


def oracle_scene(hs):
    """The oracle's view of the scene; its shadow rays traverse the BVH that
    the library's host builder makes (any-hit answers equal a brute-force
    test of every occluder)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from risltc_gb300 import api
    if len(hs.triangles):
        nodes, tris, _, _ = api.build_bvh(hs.triangles)
    else:
        nodes = tris = None
    return oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants, tris, nodes)


def cpu_sample(hs, a, seconds_target, threads=0, seed=1, count_ops=True, repeats=None, min_pixels=0):
    """Times the FP32 oracle (the reference's routines restated in C99,
    OpenMP over chunks of pixels) on pixels drawn uniformly from the frame's
    covered pixels, each shaded with the noise seed of its own position in
    frame 0 (the same computation as those pixels of the GPU's frame 0), and
    counts the algorithmic FP32 operations per pixel-sample with the
    op-counting build of the same oracle.  The sample is sized for about
    seconds_target of CPU time per render (at least min_pixels, at most the
    frame); repeats renders are timed (default: enough to fill
    seconds_target) and their median reported."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from risltc_gb300 import api
    osc = oracle_scene(hs)
    st = oracle.make_settings(candidates=a.candidates)
    rn = api.noise_constants(0)[0]
    nthreads = threads or oracle.max_threads()
    probe = _pixel_sample(hs, 256 * nthreads, seed)
    _, _, t = oracle.render_pixels(osc, st, hs.gbuffer, hs.width, hs.height, rn, probe, primitive=hs.primitive,
                                   threads=nthreads, reservoirs=False)
    want = max(int(probe.size * seconds_target / max(t, 1e-3)), min_pixels, 256)
    pixels = _pixel_sample(hs, want, seed + 1)
    if repeats is None:
        repeats = int(min(max(1, round(want / max(pixels.size, 1))), 8))
    times = []
    for _ in range(repeats):
        rgb, res, t = oracle.render_pixels(osc, st, hs.gbuffer, hs.width, hs.height, rn, pixels,
                                           primitive=hs.primitive, threads=nthreads)
        times.append(t)
    out = {"pixels": pixels, "rgb": rgb, "reservoirs": res, "samples": int(pixels.size),
           "seconds": statistics.median(times), "times": times, "threads": nthreads}
    if count_ops:
        # Counted on 1,024 sampled pixels with M candidates and with one: the
        # difference is the candidate phase, the rest the final PSA/MIS
        # shading; once more without occluders: the difference is the
        # shadow rays' BVH traversal.
        sub = _pixel_sample(hs, 1024, seed + 2)
        ops_g, m = np.ascontiguousarray(hs.gbuffer[:, sub]), sub.size
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
    (FP32, C99, OpenMP over all host threads) on a bounded pixel sample of the
    same frame per step (frame 0's noise, each pixel's own seed)."""
    if rank != 0:
        return
    hs, _ = make_workload(a)
    # The probe run stands for the warm-up; each timed step re-renders the
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
class Frame:
    """A host scene resident on the device: the context's scene, G-buffer
    and coverage tensors."""

    def __init__(self, rl, torch, ctx, hs, offsets):
        self.hs, self.offsets = hs, offsets
        self.scene = rl.Scene.from_host_scene(ctx, hs)
        if offsets is not None:
            self.scene.set_clusters(offsets)
        self.g = torch.from_numpy(hs.gbuffer).cuda()
        self.prim = torch.from_numpy(hs.primitive.view(np.int32)).cuda() if hs.primitive is not None else None
        self.samples_per_frame = int(_covered(hs).size)


def measure_throughput(a, rl, torch, ctx, fr, rank, world, local_rank, dist, steps, clocks=True):
    """Device throughput of a.spp-frame shading calls (K timed steps after W
    warm-up steps, CUDA events on the context's stream, max over ranks), the
    per-kernel times, the other numerics mode's throughput and the end-to-end
    throughput through risltc_shade_host."""
    hs = fr.hs
    s = rl.settings(candidates=a.candidates, numerics=a.numerics)
    out = torch.empty((hs.pixels, 3), dtype=torch.float32, device="cuda")
    samples_per_step = fr.samples_per_frame * a.spp
    seed = rank * 1_000_000  # each rank shades its own frames
    sampler = ClockSampler(local_rank, a.clocks_csv) if (rank == 0 and clocks) else None
    for _ in range(a.warmup):
        seed = rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, out_rgb=out,
                        primitive=fr.prim)
    ctx.check()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.profile(True)  # per-kernel CUDA events on the same stream
    launches0 = ctx.launch_count()
    if sampler:
        sampler.mark_start()
    # Inputs smaller than L2: flush it (write a 256 MB buffer) before every
    # timed step, outside that step's events.
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if hs.gbuffer.nbytes <= L2_BYTES else None
    step_events = []
    start.record(stream)
    for _ in range(steps):
        if flush is not None:
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        seed = rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, out_rgb=out,
                        primitive=fr.prim)
        if flush is not None:
            e1.record(stream)
            step_events.append((e0, e1))
    stop.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count() - launches0
    if sampler:
        sampler.mark_stop()
    if dist:
        dist.barrier()
    clock_info = sampler.stop() if sampler else None
    prof = ctx.profile(False)
    ctx.check()
    elapsed = start.elapsed_time(stop) / 1000.0
    if step_events:
        elapsed = sum(e0.elapsed_time(e1) for e0, e1 in step_events) / 1000.0
    t = torch.tensor([elapsed], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    elapsed = float(t.item())
    res = {"value": samples_per_step * world * steps / elapsed / 1e9, "ms_per_step": 1000.0 * elapsed / steps,
           "elapsed": elapsed, "samples_per_step": samples_per_step, "gpu_launches": launches, "prof": prof,
           "clocks": clock_info, "flushed": flush is not None, "rays_per_step": ctx.ray_count()}
    # The same step with the other numerics mode, for reference (exact is
    # bit-identical to the oracle; fast approximates the candidate loop).
    other = "fast" if a.numerics == "exact" else "exact"
    so = rl.settings(candidates=a.candidates, numerics=other)
    rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, so, noise_seed=seed, frames=a.spp, out_rgb=out, primitive=fr.prim)
    torch.cuda.synchronize()
    other_ms = 0.0
    ctx.profile(True)
    for _ in range(steps):
        if flush is not None:
            flush.fill_(1)
        o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        o0.record(stream)
        seed = rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, so, noise_seed=seed, frames=a.spp, out_rgb=out,
                        primitive=fr.prim)
        o1.record(stream)
        torch.cuda.synchronize()
        other_ms += o0.elapsed_time(o1)
    po = ctx.profile(False)
    pcalls = max(po["calls"], 1)
    res["other_numerics"] = {"numerics": other, "value": samples_per_step * steps / (other_ms / 1000.0) / 1e9,
                             "unit": "Gsamples/s",
                             "ms_per_launch": {k: v / pcalls for k, v in po.items() if k != "calls"}}
    # End to end through the host entry point: pinned G-buffer in, RGB out.
    res["e2e"] = None
    if not a.no_e2e:
        hg = torch.from_numpy(hs.gbuffer).pin_memory()
        hp = torch.from_numpy(hs.primitive.view(np.int32)).pin_memory() if hs.primitive is not None else None
        ho = torch.empty((hs.pixels, 3), dtype=torch.float32).pin_memory()
        hgn, hon = hg.numpy(), ho.numpy()
        hpn = hp.numpy().view(np.uint32) if hp is not None else None
        for _ in range(max(1, a.warmup // 2)):
            rl.shade_host(ctx, fr.scene, hgn, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, primitive=hpn,
                          out=hon)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            rl.shade_host(ctx, fr.scene, hgn, hs.width, hs.height, s, noise_seed=seed, frames=a.spp, primitive=hpn,
                          out=hon)
            seed += a.spp
        te = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device="cuda")
        if dist:
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
        res["e2e"] = {"value": samples_per_step * world * steps / float(te.item()) / 1e9, "unit": "Gsamples/s",
                      "h2d_bytes_per_step": int(hs.gbuffer.nbytes + (hs.primitive.nbytes if hs.primitive is not None
                                                                    else 0)),
                      "d2h_bytes_per_step": int(hs.pixels * 3 * 4)}
    return res


def kernel_table(prof, samples_per_step, info, fp32_peak, peaks):
    """Per-kernel ms per launch (CUDA events) and, with the op counts of the
    CPU leg, achieved FP32 work against the FP32 peak; the traversal's
    node and triangle bytes (served from L1/L2) against its time."""
    calls = max(prof["calls"], 1)
    # One launch of each kernel per step (all spp frames in one call).
    kernels = {"ris_candidates_binned_kernel": {"ms_per_launch": prof["candidates"] / calls},
               "ris_sample_kernel": {"ms_per_launch": prof["shade"] / calls},
               "light_bucket_scan_kernel + shadow_scatter_kernel": {"ms_per_launch": prof["ray_sort"] / calls},
               "shadow_trace_kernel": {"ms_per_launch": prof["shadow_trace"] / calls},
               "ris_resolve_kernel": {"ms_per_launch": prof["resolve"] / calls}}
    if info and "flops_per_sample" in info:
        kernels["ris_candidates_binned_kernel"]["flops_per_sample"] = info["candidate_flops_per_sample"]
        kernels["ris_sample_kernel"]["flops_per_sample"] = info["shade_flops_per_sample"]
        kernels["shadow_trace_kernel"]["flops_per_sample"] = info["trace_flops_per_sample"]
        kernels["light_bucket_scan_kernel + shadow_scatter_kernel"]["flops_per_sample"] = 0.0
        kernels["ris_resolve_kernel"]["flops_per_sample"] = 0.0
        tk = kernels["shadow_trace_kernel"]
        tk["node_triangle_bytes_per_sample"] = info["trace_bytes_per_sample"]
        tk["node_triangle_gbs"] = (tk["node_triangle_bytes_per_sample"] * samples_per_step
                                   / (tk["ms_per_launch"] / 1e3) / 1e9 if tk["ms_per_launch"] > 0 else 0.0)
        tk["node_triangle_note"] = ("BVH node and triangle bytes the traversal reads (oracle-counted on the identical "
                                    "BVH), served from L1 and L2; DRAM bytes are in dram_gbs")
        for k in kernels.values():
            k["achieved_tflops"] = (k["flops_per_sample"] * samples_per_step / (k["ms_per_launch"] / 1e3) / 1e12
                                    if k["ms_per_launch"] > 0 else 0.0)
            k["frac"] = k["achieved_tflops"] / fp32_peak
    return kernels


def attach_dram(kernels, workload, samples_per_step, peaks):
    for name, k in kernels.items():
        traffic, source = measured_traffic(name, workload, samples_per_step) if workload else (None, None)
        if traffic is not None and k["ms_per_launch"] > 0:
            k["dram_bytes_per_launch"] = traffic
            k["dram_gbs"] = traffic / (k["ms_per_launch"] / 1e3) / 1e9
            if peaks.get("hbm_gbs"):
                k["dram_frac_of_hbm"] = k["dram_gbs"] / peaks["hbm_gbs"]
            k["dram_source"] = source


def rates_of(a, thr, kernels):
    """Candidates per second (M per pixel-sample) and shadow rays per second
    (the rays of the last timed call, which risltc_ctx_ray_count reports)
    over the step and over the trace kernel's own time."""
    rays = thr.get("rays_per_step") or 0
    trace = kernels.get("shadow_trace_kernel", {}).get("ms_per_launch")
    return {"gcandidates_per_s": thr["value"] * a.candidates, "shadow_rays_per_step": rays,
            "grays_per_s_step": rays / (thr["ms_per_step"] / 1e3) / 1e9 if rays else None,
            "grays_per_s_trace_kernel": rays / (trace / 1e3) / 1e9 if rays and trace else None}


def roofline_of(kernels, fp32_peak, flops_per_sample, samples_per_step, ms_per_step, sms, sm_max, workload):
    dominant = max(kernels, key=lambda k: kernels[k]["ms_per_launch"])
    d = kernels[dominant]
    if "achieved_tflops" not in d:
        return None
    traffic, source = measured_traffic(dominant, workload, samples_per_step) if workload else (None, None)
    return {"bound": "fp32", "achieved": d["achieved_tflops"], "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": d["frac"], "traffic": traffic, "traffic_source": source, "kernel": dominant,
            "flops_per_sample": d["flops_per_sample"],
            "whole_step_frac": flops_per_sample * samples_per_step / (ms_per_step / 1e3) / 1e12 / fp32_peak,
            # Exact numerics never contracts a multiply and an add (its
            # results equal an oracle without fused operations), so one FP32
            # instruction performs at most one of the counted operations.
            "unfused_peak": fp32_peak / 2, "frac_of_unfused_peak": 2 * d["frac"],
            "peak_source": "derived: 2 x 128 FP32 lanes x %d SMs x %.0f MHz (max SM clock of MEASURED_PEAKS.json); "
                           "no measured FP32 peak exists" % (sms, sm_max)}


def parity_check(rl, torch, ctx, fr, a, info):
    """The GPU's frame 0 (one-frame call, noise seed 0) against the oracle's
    pixels of the CPU-baseline sample: pixels whose colour differs in any
    bit, and reservoirs whose chosen light, w_sum or p_hat differ."""
    hs = fr.hs
    out = torch.zeros((hs.pixels, 3), dtype=torch.float32, device="cuda")
    res = torch.zeros((hs.pixels, 4), dtype=torch.int32, device="cuda")
    rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, rl.settings(candidates=a.candidates, numerics="exact"),
             noise_seed=0, frames=1, out_rgb=out, reservoirs=res, primitive=fr.prim)
    ctx.check()
    idx = torch.from_numpy(info["pixels"].astype(np.int64)).cuda()
    got, r = out[idx].cpu().numpy(), res[idx].cpu().numpy()
    want, wres = info["rgb"], info["reservoirs"]
    wp = r[:, 1:3].copy().view(np.float32)
    bad_rgb = np.any(got != want, axis=1)
    bad_res = ((r[:, 0] != wres["light_index"]) | (wp[:, 0] != wres["w_sum"].astype(np.float32))
               | (wp[:, 1] != wres["sample_value"].astype(np.float32)))
    return {"pixels": int(idx.numel()), "mismatches": int(bad_rgb.sum()), "reservoir_mismatches": int(bad_res.sum()),
            "numerics": "exact", "frame": "frame 0 (noise seed 0), 1 spp, every pixel with its own seed",
            "oracle": "FP32 C99 restatement of the reference's routines"}


def measure_equal_mse(a, rl, torch, ctx, fr, local_rank):
    """Device time to equal MSE, learned cluster proposal vs plain RIS.

    Reference: a.reference_spp spp of plain RIS accumulated in FP64 on the
    GPU.  The learned proposal's model trains online for a.train_frames
    frames first (1 spp each, every a.train_stride-th pixel).  Then each
    method renders a.mse_spp spp four times with fresh noise and its MSE
    against the reference is measured, and its device time per frame (CUDA
    events over a.mse_steps calls of a.mse_spp frames each, training off).
    MSE falls as 1 / spp for these unbiased estimators, so the time to reach
    plain RIS's a.mse_spp-spp MSE is ms_per_frame * spp * MSE(method) /
    MSE(plain)."""
    hs = fr.hs
    k = fr.offsets.size - 1
    model = rl.Model(ctx, k, seed=2)
    model.set_input_transform((0.0, 0.0, 1.0), 6.0)
    fr.scene.set_model(model)
    covered = torch.from_numpy(hs.primitive == 0).cuda() if hs.primitive is not None else None
    plain = rl.settings(candidates=a.candidates)
    clusters = rl.settings(candidates=a.candidates, proposal="clusters", proposal_uniform_fraction=a.uniform_fraction)
    learned = rl.settings(candidates=a.candidates, proposal="learned", proposal_uniform_fraction=a.uniform_fraction)
    acc = torch.zeros((hs.pixels, 3), dtype=torch.float64, device="cuda")
    seed = 10_000_000
    for _ in range(a.reference_spp // 16):
        seed = rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, plain, noise_seed=seed, frames=16, accum=acc,
                        primitive=fr.prim)
    reference = acc / (16 * (a.reference_spp // 16))
    ctx.check()
    model.set_training(True, learning_rate=a.learning_rate, pixel_stride=a.train_stride)
    model.set_training_flags(cuda_cores=a.train_on_cuda_cores)
    model.set_target_mix(a.shadowed_target)
    out = torch.empty((hs.pixels, 3), dtype=torch.float32, device="cuda")
    seed = 20_000_000
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(a.train_frames):
        seed = rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, learned, noise_seed=seed, frames=1, out_rgb=out,
                        primitive=fr.prim)
    t1.record()
    torch.cuda.synchronize()
    train_ms = t0.elapsed_time(t1) / max(a.train_frames, 1)
    model.set_training(False)
    results = {}
    runs = [("plain", plain), ("clusters", clusters), ("learned", learned)]
    for m in [int(x) for x in a.sweep_candidates.split(",") if x.strip()]:
        if m != a.candidates:
            runs += [("%s_m%d" % (name, m), rl.copy_settings(st, candidate_count=m)) for name, st in runs[:3]]
    sampler = ClockSampler(local_rank, None)
    sampler.mark_start()
    timed_ms = 0.0
    for name, s in runs:
        mses = []
        for rep in range(4):
            rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, s, noise_seed=30_000_000 + 1000 * rep,
                     frames=a.mse_spp, out_rgb=out, primitive=fr.prim)
            d = (out.double() - reference) ** 2
            if covered is not None:
                d = d[covered]
            mses.append(float(d.mean()))
        for _ in range(a.warmup):
            rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, s, noise_seed=seed, frames=a.mse_spp, out_rgb=out,
                     primitive=fr.prim)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(a.mse_steps):
            rl.shade(ctx, fr.scene, fr.g, hs.width, hs.height, s, noise_seed=40_000_000 + a.mse_spp * i,
                     frames=a.mse_spp, out_rgb=out, primitive=fr.prim)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        timed_ms += ms
        results[name] = {"mse_at_spp": statistics.mean(mses), "ms_per_frame": ms / (a.mse_spp * a.mse_steps),
                         "candidates": int(s.candidate_count)}
    sampler.mark_stop()
    clocks = sampler.stop()
    ctx.check()
    fr.scene.set_model(None)
    model.close()
    base = results["plain"]
    for r in results.values():
        r["ms_to_plain_mse"] = r["ms_per_frame"] * a.mse_spp * r["mse_at_spp"] / base["mse_at_spp"]
    best = {}
    for method in ("plain", "clusters", "learned"):
        keys = [key for key in results if key == method or key.startswith(method + "_m")]
        key = min(keys, key=lambda q: results[q]["ms_to_plain_mse"])
        best[method] = {"run": key, "candidates": results[key]["candidates"],
                        "ms_to_plain_mse": results[key]["ms_to_plain_mse"]}
    return {
        "metric": "ms/frame to equal MSE, learned-proposal vs plain RIS (%dx%d, %d lights)"
                  % (hs.width, hs.height, hs.light_count),
        "unit": "ms", "higher_is_better": False,
        "learned_ms_to_plain_mse": best["learned"]["ms_to_plain_mse"],
        "plain_ms_to_equal_mse": base["ms_to_plain_mse"],
        "clusters_ms_to_plain_mse": best["clusters"]["ms_to_plain_mse"],
        "speedup_vs_plain": base["ms_to_plain_mse"] / results["learned"]["ms_to_plain_mse"],
        "speedup_best_vs_plain": base["ms_to_plain_mse"] / best["learned"]["ms_to_plain_mse"],
        "speedup_best_vs_best_plain": best["plain"]["ms_to_plain_mse"] / best["learned"]["ms_to_plain_mse"],
        "learned_vs_heuristic": best["clusters"]["ms_to_plain_mse"] / best["learned"]["ms_to_plain_mse"],
        "best_candidate_count": best,
        "methods": results,
        "config": {"protocol": "MSE at %d spp against a %d-spp FP64 plain-RIS reference (4 repetitions with fresh "
                               "noise); device time of %d calls of %d frames per method; plain RIS at M=%d is the "
                               "MSE level" % (a.mse_spp, a.reference_spp, a.mse_steps, a.mse_spp, a.candidates),
                   "clusters": k, "train_frames": a.train_frames, "train_ms_per_frame": train_ms,
                   "learning_rate": a.learning_rate, "train_stride": a.train_stride,
                   "uniform_fraction": a.uniform_fraction,
                   "training": ("cuda cores fp32" if a.train_on_cuda_cores else "tensor cores bf16 (tcgen05)"),
                   "shadowed_target": a.shadowed_target},
        "timed_ms": timed_ms,
        "clocks": clocks,
    }


def base_line(a, world, thr):
    return {"metric": metric_name(a), "value": thr["value"], "unit": "Gsamples/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": thr["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generators)"}


def config_of(a, hs, thr, world):
    return {"workload": workload_name(a), "width": hs.width, "height": hs.height, "lights": hs.light_count,
            "clusters": a.clusters, "triangles": int(hs.triangles.shape[0]), "candidates": a.candidates,
            "spp": a.spp, "numerics": a.numerics, "samples_per_step": thr["samples_per_step"],
            "l2": ("inputs smaller than L2 (G-buffer %.0f MB < 129 MB): L2 flushed (256 MB written) before every "
                   "timed step, outside its events" if thr["flushed"] else
                   "inputs larger than L2 (G-buffer %.0f MB > 129 MB)") % (hs.gbuffer.nbytes / 1e6),
            "parallelism": "one frame per GPU" if world > 1 else "single GPU"}


def run_ours(a, rank, world, local_rank):
    """--workload headline (default) and throughput."""
    import torch
    import risltc_gb300 as rl
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    hs, offsets = make_workload(a, seed=0)
    ctx = rl.Context(local_rank)
    fr = Frame(rl, torch, ctx, hs, offsets)
    thr = measure_throughput(a, rl, torch, ctx, fr, rank, world, local_rank, dist, a.steps)
    single = world == 1 and rank == 0
    info = {}
    parity = None
    if single and not a.no_cpu_baseline:
        info = cpu_sample(hs, a, a.cpu_seconds, min_pixels=a.parity_pixels)
        parity = parity_check(rl, torch, ctx, fr, a, info)
    equal_mse = None
    if single and a.workload == "headline" and not a.no_equal_mse and offsets is not None:
        equal_mse = measure_equal_mse(a, rl, torch, ctx, fr, local_rank)
    fr.scene.close()
    config2 = None
    if single and a.workload == "headline" and not a.no_config2:
        b = parse(["--workload", "throughput", "--steps", str(min(a.steps, 10)), "--warmup", str(a.warmup),
                   "--no-e2e", "--numerics", a.numerics])
        hs2, _ = make_workload(b)
        fr2 = Frame(rl, torch, ctx, hs2, None)
        t2 = measure_throughput(b, rl, torch, ctx, fr2, rank, world, local_rank, None, b.steps, clocks=False)
        fr2.scene.close()
        calls = max(t2["prof"]["calls"], 1)
        config2 = {"workload": workload_name(b), "value": t2["value"], "unit": "Gsamples/s",
                   "ms_per_step": t2["ms_per_step"], "steps": b.steps,
                   "other_numerics": t2["other_numerics"],
                   "ms_per_launch": {k: v / calls for k, v in t2["prof"].items() if k != "calls"}}
    ctx.close()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks = measured_peaks()
    props = torch.cuda.get_device_properties(local_rank)
    sms = props.multi_processor_count
    sm_max = peaks.get("sm_max_mhz") or (thr["clocks"] or {}).get("sm_max_mhz") or 2070.0
    fp32_peak = 2.0 * 128 * sms * sm_max * 1e6 / 1e12  # TFLOP/s, 128 FP32 lanes per SM
    kernels = kernel_table(thr["prof"], thr["samples_per_step"], info, fp32_peak, peaks)
    attach_dram(kernels, traffic_key(a), thr["samples_per_step"], peaks)
    roofline = None
    if info:
        roofline = roofline_of(kernels, fp32_peak, info["flops_per_sample"], thr["samples_per_step"],
                               thr["ms_per_step"], sms, sm_max, traffic_key(a))
        other = thr["other_numerics"]
        oms = other.get("ms_per_launch", {}).get("candidates", 0.0)
        if roofline and oms > 0 and roofline["kernel"] == "ris_candidates_binned_kernel":
            # The same kernel and op count in the other numerics mode.
            ach = roofline["flops_per_sample"] * thr["samples_per_step"] / (oms / 1e3) / 1e12
            roofline["other_numerics"] = {"numerics": other["numerics"], "ms_per_launch": oms, "achieved": ach,
                                          "frac": ach / fp32_peak}
    cpu = None
    if info:
        cpu = {"value": info["samples"] / info["seconds"] / 1e9, "unit": "Gsamples/s", "cores": info["threads"],
               "kind": "port", "sample": "%d pixels drawn uniformly from the same frame, frame 0 at 1 spp (each "
                                         "pixel's own noise seed), FP32 oracle (C99, OpenMP), median of %d renders"
                                         % (info["samples"], len(info["times"]))}
    line = base_line(a, world, thr)
    line.update({
        "config": config_of(a, hs, thr, world),
        "gpu_launches": thr["gpu_launches"],
        "rates": rates_of(a, thr, kernels),
        "kernels": kernels,
        "other_numerics": thr["other_numerics"],
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": thr["e2e"],
        "parity": parity,
        "equal_mse": equal_mse,
        "config2": config2,
        "clocks": thr["clocks"],
    })
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_equal_mse(a):
    """--workload equal-mse: the equal-MSE comparison alone, as its own line."""
    import torch
    import risltc_gb300 as rl
    hs, offsets = make_workload(a, seed=0)
    if offsets is None:
        raise SystemExit("equal-mse needs light clusters (--clusters > 0)")
    ctx = rl.Context(0)
    fr = Frame(rl, torch, ctx, hs, offsets)
    eq = measure_equal_mse(a, rl, torch, ctx, fr, 0)
    fr.scene.close()
    ctx.close()
    line = {"metric": eq["metric"] + "; Gsamples/s", "value": eq["learned_ms_to_plain_mse"], "unit": "ms",
            "higher_is_better": False, "n_gpus": 1, "steps": a.mse_steps, "warmup": a.warmup,
            "dtype": "f32 (MLP bf16/fp32)", "data": "synthetic",
            "config": dict(eq["config"], workload="equal MSE: " + workload_name(a)),
            "gsamples_per_s": {key: fr.samples_per_frame / (v["ms_per_frame"] / 1e3) / 1e9
                               for key, v in eq["methods"].items()}}
    line.update({k: v for k, v in eq.items() if k not in ("config", "metric", "unit", "higher_is_better")})
    print(json.dumps(line), flush=True)


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
    launches0 = ctx.launch_count()
    with torch.cuda.graph(graph, stream=stream):
        rl.shade_batch(ctx, items)
    launches_per_batch = ctx.launch_count() - launches0
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
        "config": {"workload": "batch of %d scenes in one CUDA-graph replay of risltc_shade_batch (%d kernels per "
                               "replay)" % (len(hss), launches_per_batch),
                   "scenes": [{"width": hs.width, "height": hs.height, "lights": hs.light_count,
                               "triangles": int(hs.triangles.shape[0])} for hs in hss],
                   "candidates": a.batch_candidates, "numerics": a.numerics, "samples_per_step": samples_per_step,
                   "tile": tile, "autotune_ms_per_batch": tile_ms,
                   "l2": "inputs larger than L2 (G-buffers %.0f MB > 129 MB)"
                         % (sum(hs.gbuffer.nbytes for hs in hss) / 1e6)},
        "gpu_launches": launches_per_batch * a.steps,
        "roofline": None,
        "roofline_note": "each kernel of the batch covers all items' work (one launch per phase); the per-kernel "
                         "roofline is reported by "
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
