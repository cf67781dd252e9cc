"""Batched shading (risltc_shade_batch): 16 frames of the plane-of-quads form
(G-buffer on z = 0, quads above it, optional occluders) with mixed
resolutions, light counts and occluder counts, shaded in one call and in one
captured CUDA graph, equal bit for bit to one risltc_shade call per frame.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def batch_scenes(count=16, seed=5):
    import risltc_gb300 as rl
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        # Log-uniform sizes, light counts and occluder counts, scaled down from
        # the 256^2..1080p, 16..8192-light, 10k..500k-triangle batch workload.
        w = int(np.exp(rng.uniform(np.log(24), np.log(160))))
        h = int(np.exp(rng.uniform(np.log(16), np.log(96))))
        lights = int(np.exp(rng.uniform(np.log(16), np.log(512))))
        tris = 0 if i % 3 == 0 else int(np.exp(rng.uniform(np.log(500), np.log(5000))))
        out.append(rl.scenes.plane_of_quads(w, h, lights, seed=seed * 100 + i, triangles=tris))
    return out


def test_batch_and_graph_equal_single_calls(gpu):
    import torch
    import risltc_gb300 as rl
    stream = torch.cuda.Stream()
    ctx = rl.Context(0, stream=stream.cuda_stream)
    hss = batch_scenes()
    scenes = [rl.Scene.from_host_scene(ctx, hs) for hs in hss]
    s = rl.settings(candidates=8)
    items, singles = [], []
    with torch.cuda.stream(stream):
        for k, (hs, sc) in enumerate(zip(hss, scenes)):
            g = torch.from_numpy(hs.gbuffer).cuda()
            frames = 1 + k % 3
            one = torch.zeros((hs.pixels, 3), dtype=torch.float32, device="cuda")
            rl.shade(ctx, sc, g, hs.width, hs.height, s, noise_seed=7 * k, frames=frames, out_rgb=one)
            singles.append(one)
            items.append(dict(scene=sc, gbuffer=g, width=hs.width, height=hs.height, settings=s, noise_seed=7 * k,
                              frames=frames, out_rgb=torch.full((hs.pixels, 3), -1.0, device="cuda")))
        seeds = rl.shade_batch(ctx, items)
    ctx.check()
    assert seeds == [7 * k + 1 + k % 3 for k in range(len(items))]
    for it, one in zip(items, singles):
        assert torch.equal(it["out_rgb"], one)
    # The same batch captured into one graph and replayed.
    for it in items:
        it["out_rgb"].fill_(-1.0)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        rl.shade_batch(ctx, items)
    graph.replay()
    torch.cuda.synchronize()
    ctx.check()
    for it, one in zip(items, singles):
        assert torch.equal(it["out_rgb"], one)
    for sc in scenes:
        sc.close()
    ctx.close()


def test_batch_rejects_a_bad_item_before_any_work(gpu):
    import torch
    import risltc_gb300 as rl
    ctx = rl.Context(0)
    hs = rl.scenes.plane_of_quads(32, 32, 16, seed=1)
    sc = rl.Scene.from_host_scene(ctx, hs)
    g = torch.from_numpy(hs.gbuffer).cuda()
    out = torch.full((hs.pixels, 3), -1.0, device="cuda")
    good = dict(scene=sc, gbuffer=g, width=hs.width, height=hs.height, settings=rl.settings(), out_rgb=out)
    bad = dict(good, settings=rl.settings(candidates=0))
    with pytest.raises(rl.RisltcError):
        rl.shade_batch(ctx, [good, bad])
    torch.cuda.synchronize()
    assert torch.all(out == -1.0)
    sc.close()
    ctx.close()


@pytest.mark.parametrize("tile", ["32x8", "16x4"])
def test_whole_batch_launches_equal_single_calls(gpu, tile):
    """20 shadowed frames of mixed sizes, light and occluder counts in the
    default configuration: risltc_shade_batch runs one launch per phase for
    each group of 16 items (6 kernels per group, counted by the context), and
    every item's image, FP64 sums and reservoirs equal its own risltc_shade
    call bit for bit, also when replayed from a captured graph."""
    import torch
    import risltc_gb300 as rl
    rng = np.random.default_rng(9)
    hss = []
    for i in range(20):
        w = int(np.exp(rng.uniform(np.log(24), np.log(160))))
        h = int(np.exp(rng.uniform(np.log(16), np.log(96))))
        lights = int(np.exp(rng.uniform(np.log(16), np.log(512))))
        tris = int(np.exp(rng.uniform(np.log(300), np.log(5000))))
        hss.append(rl.scenes.plane_of_quads(w, h, lights, seed=900 + i, triangles=tris))
    stream = torch.cuda.Stream()
    ctx = rl.Context(0, stream=stream.cuda_stream)
    scenes = [rl.Scene.from_host_scene(ctx, hs) for hs in hss]
    s = rl.settings(candidates=8, tile=tile)
    items, singles = [], []
    with torch.cuda.stream(stream):
        for k, (hs, sc) in enumerate(zip(hss, scenes)):
            g = torch.from_numpy(hs.gbuffer).cuda()
            frames = 1 + k % 2
            want = (torch.zeros((hs.pixels, 3), dtype=torch.float32, device="cuda"),
                    torch.zeros((hs.pixels, 3), dtype=torch.float64, device="cuda"),
                    torch.zeros((hs.pixels, 4), dtype=torch.int32, device="cuda"))
            rl.shade(ctx, sc, g, hs.width, hs.height, s, noise_seed=11 * k, frames=frames, out_rgb=want[0],
                     accum=want[1], reservoirs=want[2])
            singles.append(want)
            items.append(dict(scene=sc, gbuffer=g, width=hs.width, height=hs.height, settings=s, noise_seed=11 * k,
                              frames=frames, out_rgb=torch.full((hs.pixels, 3), -1.0, device="cuda"),
                              accum=torch.zeros((hs.pixels, 3), dtype=torch.float64, device="cuda"),
                              reservoirs=torch.zeros((hs.pixels, 4), dtype=torch.int32, device="cuda")))
        before = ctx.launch_count()
        seeds = rl.shade_batch(ctx, items)
        assert ctx.launch_count() - before == 2 * 6
    ctx.check()
    assert seeds == [11 * k + 1 + k % 2 for k in range(len(items))]

    def check():
        for it, (rgb, acc, res) in zip(items, singles):
            assert torch.equal(it["out_rgb"], rgb)
            assert torch.equal(it["accum"], acc)
            assert torch.equal(it["reservoirs"], res)
    check()
    for it in items:
        it["out_rgb"].fill_(-1.0)
        it["accum"].zero_()
        it["reservoirs"].zero_()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        rl.shade_batch(ctx, items)
    graph.replay()
    torch.cuda.synchronize()
    ctx.check()
    check()
    for sc in scenes:
        sc.close()
    ctx.close()


def test_single_call_graph_replay_equals_direct_call(gpu):
    """One risltc_shade call of the default configuration (shadow rays
    through the ray queue, two frames, FP64 sums and reservoirs), captured
    into a CUDA graph after a first call has sized the scratch: every replay
    equals the same call made directly, bit for bit."""
    import torch
    import risltc_gb300 as rl
    hs = rl.scenes.plane_of_quads(160, 96, 200, seed=31, triangles=3000)
    stream = torch.cuda.Stream()
    ctx = rl.Context(0, stream=stream.cuda_stream)
    sc = rl.Scene.from_host_scene(ctx, hs)
    s = rl.settings(candidates=16)

    def buffers():
        return (torch.full((hs.pixels, 3), -1.0, dtype=torch.float32, device="cuda"),
                torch.zeros((hs.pixels, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((hs.pixels, 4), dtype=torch.int32, device="cuda"))
    with torch.cuda.stream(stream):
        g = torch.from_numpy(hs.gbuffer).cuda()
        want = buffers()
        assert rl.shade(ctx, sc, g, hs.width, hs.height, s, noise_seed=9, frames=2, out_rgb=want[0], accum=want[1],
                        reservoirs=want[2]) == 11
        got = buffers()
    torch.cuda.synchronize()
    ctx.check()
    assert ctx.ray_count() > 0
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        rl.shade(ctx, sc, g, hs.width, hs.height, s, noise_seed=9, frames=2, out_rgb=got[0], accum=got[1],
                 reservoirs=got[2])
    for _ in range(2):
        got[0].fill_(-1.0)
        got[1].zero_()
        got[2].zero_()
        graph.replay()
        torch.cuda.synchronize()
        ctx.check()
        for a, b in zip(got, want):
            assert torch.equal(a, b)
    sc.close()
    ctx.close()
