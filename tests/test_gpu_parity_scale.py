"""Parity of the CUDA path with the oracle at the benchmark workloads' full sizes.

Three frames at the sizes the benchmark runs:

* plane of quads: 256x256 G-buffer on z = 0, 64 quad lights, M = 8, 1 spp,
  unshadowed (every pixel compared);
* shadowed heightfield: 1920x1080, 1024 lights of 3-8 vertices, 200k occluder
  triangles (about 550k split-clipped BVH references), M = 32, 4 spp;
* many lights: 1920x1080 heightfield, 16,384 lights of 3-8 vertices listed in
  256 k-means clusters, 1M occluders (a BVH larger than the 129 MB L2),
  M = 32, plain RIS and the heuristic cluster proposal.

The GPU shades the whole frame through the C ABI; the oracle shades a uniform
sample of its covered pixels, each with the noise seed of its own position
(noise_utility.glsl:77-84), so the two pixels are the same computation.  The
oracle traces shadow rays by brute force over every occluder: the GPU's BVH
(split-clipped references, deep stacks, many-reference leaves, nodes beyond
L2) is checked against the plain definition of visibility.  Exact numerics:
colour, chosen light, w_sum and p_hat equal bit for bit, per frame, and the
multi-frame mean equals the FP32 mean of the oracle's frames.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SAMPLE_PIXELS = 4096


@pytest.fixture(scope="module")
def rl(gpu):
    import torch
    import risltc_gb300 as rl
    ctx = rl.Context(0)
    yield rl, ctx, torch
    ctx.close()


def sample_pixels(hs, count, seed):
    valid = np.flatnonzero(hs.primitive == 0) if hs.primitive is not None else np.arange(hs.pixels)
    if count >= valid.size:
        return valid.astype(np.uint32)
    return np.sort(np.random.default_rng(seed).choice(valid, count, replace=False)).astype(np.uint32)


def compare_frames(rl_tuple, hs, gpu_settings, oracle_settings_for, frames, pixels, scene=None, osc=None):
    """Shades `frames` single frames (noise seeds 0..frames-1) and one
    multi-frame call on the GPU, the same frames on the oracle at `pixels`;
    asserts bit equality.  oracle_settings_for(frame) gives the oracle's
    settings of that frame."""
    rlm, ctx, torch = rl_tuple
    own_scene = scene is None
    if own_scene:
        scene = rlm.Scene.from_host_scene(ctx, hs)
    if osc is None:
        tris = oracle.triangles_v0e1e2(hs.triangles) if len(hs.triangles) else None
        osc = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants, tris)
    g = torch.from_numpy(hs.gbuffer).cuda()
    prim = None if hs.primitive is None else torch.from_numpy(hs.primitive.view(np.int32)).cuda()
    out = torch.zeros((hs.pixels, 3), dtype=torch.float32, device="cuda")
    res = torch.zeros((hs.pixels, 4), dtype=torch.int32, device="cuda")
    idx = torch.from_numpy(pixels.astype(np.int64)).cuda()
    oracle_frames = []
    for f in range(frames):
        rlm.shade(ctx, scene, g, hs.width, hs.height, gpu_settings, noise_seed=f, frames=1, out_rgb=out,
                  reservoirs=res, primitive=prim)
        ctx.check()
        got = out[idx].cpu().numpy()
        r = res[idx].cpu().numpy()
        want, wres, _ = oracle.render_pixels(osc, oracle_settings_for(f), hs.gbuffer, hs.width, hs.height,
                                             rlm.noise_constants(f)[0], pixels, primitive=hs.primitive)
        oracle_frames.append(want)
        bad = np.any(got != want, axis=1)
        assert not bad.any(), "frame %d: %d of %d sampled pixels differ (first %s)" % (
            f, bad.sum(), pixels.size, pixels[np.flatnonzero(bad)[:5]])
        assert np.array_equal(r[:, 0], wres["light_index"]), "frame %d: chosen lights differ" % f
        wp = r[:, 1:3].copy().view(np.float32)
        assert np.array_equal(wp[:, 0], wres["w_sum"].astype(np.float32)), "frame %d: w_sum differs" % f
        assert np.array_equal(wp[:, 1], wres["sample_value"].astype(np.float32)), "frame %d: p_hat differs" % f
    if frames > 1:
        rlm.shade(ctx, scene, g, hs.width, hs.height, gpu_settings, noise_seed=0, frames=frames, out_rgb=out,
                  primitive=prim)
        ctx.check()
        total = oracle_frames[0].copy()
        for fr in oracle_frames[1:]:
            total = total + fr
        assert np.array_equal(out[idx].cpu().numpy(), total * np.float32(1.0 / frames))
    if own_scene:
        scene.close()
    return oracle_frames


def test_plane_of_quads_256_full_frame(rl):
    import risltc_gb300 as rlm
    hs = rlm.scenes.plane_of_quads(256, 256, 64, seed=0)
    pixels = np.arange(hs.pixels, dtype=np.uint32)
    compare_frames(rl, hs, rlm.settings(candidates=8), lambda f: oracle.make_settings(candidates=8), 1, pixels)


@pytest.fixture(scope="module")
def shadowed_1080p():
    import risltc_gb300 as rlm
    return rlm.scenes.heightfield(1920, 1080, light_count=1024, triangle_count=200_000, seed=0, vertex_counts=(3, 8))


def test_shadowed_1080p_1024_lights_200k_occluders(rl, shadowed_1080p):
    import risltc_gb300 as rlm
    hs = shadowed_1080p
    frames = compare_frames(rl, hs, rlm.settings(candidates=32), lambda f: oracle.make_settings(candidates=32), 4,
                            sample_pixels(hs, SAMPLE_PIXELS, 11))
    # The sample holds both lit pixels and pixels whose light is occluded or
    # faces away.
    lit = (frames[0].sum(1) > 0).mean()
    assert 0.1 < lit < 0.99


def test_shadowed_1080p_fast_numerics_within_tolerance(rl, shadowed_1080p):
    """Fast numerics at full size: light choice agrees on 99.9% of the sampled
    pixels, and where it agrees the estimate is within 1e-2 relative for 99%
    of them (the tolerance of the small-scene fast-numerics test)."""
    rlm, ctx, torch = rl
    hs = shadowed_1080p
    pixels = sample_pixels(hs, SAMPLE_PIXELS, 12)
    scene = rlm.Scene.from_host_scene(ctx, hs)
    g = torch.from_numpy(hs.gbuffer).cuda()
    prim = torch.from_numpy(hs.primitive.view(np.int32)).cuda()
    out = torch.zeros((hs.pixels, 3), dtype=torch.float32, device="cuda")
    res = torch.zeros((hs.pixels, 4), dtype=torch.int32, device="cuda")
    rlm.shade(ctx, scene, g, hs.width, hs.height, rlm.settings(candidates=32, numerics="fast"), noise_seed=0,
              out_rgb=out, reservoirs=res, primitive=prim)
    ctx.check()
    scene.close()
    idx = torch.from_numpy(pixels.astype(np.int64)).cuda()
    got, r = out[idx].cpu().numpy(), res[idx].cpu().numpy()
    tris = oracle.triangles_v0e1e2(hs.triangles)
    osc = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants, tris)
    want, wres, _ = oracle.render_pixels(osc, oracle.make_settings(candidates=32), hs.gbuffer, hs.width, hs.height,
                                         rlm.noise_constants(0)[0], pixels, primitive=hs.primitive)
    agree = r[:, 0] == wres["light_index"]
    assert agree.mean() >= 0.999
    m = agree & (want.sum(1) > 0)
    rel = np.abs(got[m].sum(1) - want[m].sum(1)) / want[m].sum(1)
    assert np.quantile(rel, 0.99) <= 1e-2


@pytest.fixture(scope="module")
def many_lights_1080p():
    import risltc_gb300 as rlm
    hs0 = rlm.scenes.heightfield(1920, 1080, light_count=16384, triangle_count=1_000_000, seed=0,
                                 vertex_counts=(3, 8))
    hs, offsets = rlm.scenes.cluster_lights(hs0, 256, seed=1)
    bounds, power = rlm.scenes.cluster_summaries(hs.lights, hs.max_vertex_count, offsets)
    return hs, offsets, bounds, power


def test_many_lights_1080p_16k_lights_1m_occluders(rl, many_lights_1080p):
    """Plain RIS and the heuristic cluster proposal on the 16K-light scene
    (lights listed cluster by cluster, 1M occluders)."""
    rlm, ctx, torch = rl
    hs, offsets, bounds, power = many_lights_1080p
    scene = rlm.Scene.from_host_scene(ctx, hs)
    scene.set_clusters(offsets)
    tris = oracle.triangles_v0e1e2(hs.triangles)
    osc = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants, tris)
    osc.set_clusters(offsets, bounds, power)
    pixels = sample_pixels(hs, SAMPLE_PIXELS, 13)
    compare_frames(rl, hs, rlm.settings(candidates=32), lambda f: oracle.make_settings(candidates=32), 1, pixels,
                   scene=scene, osc=osc)
    compare_frames(rl, hs, rlm.settings(candidates=32, proposal="clusters", proposal_uniform_fraction=0.05),
                   lambda f: oracle.make_settings(candidates=32, proposal=True, proposal_uniform_fraction=0.05,
                                                  random_number_proposal=rlm.noise_constants(f)[1]),
                   2, sample_pixels(hs, SAMPLE_PIXELS // 2, 14), scene=scene, osc=osc)
    scene.close()


def test_many_lights_shadow_queries_match_brute_force(rl, many_lights_1080p):
    """Any-hit queries through the 1M-occluder BVH (larger than L2) from the
    frame's shading points toward random light vertices, against brute force."""
    import ctypes
    rlm, ctx, torch = rl
    hs = many_lights_1080p[0]
    rng = np.random.default_rng(15)
    pixels = sample_pixels(hs, 8192, 16)
    n = pixels.size
    origin = hs.gbuffer[0:3, pixels].T
    light = rng.integers(0, hs.light_count, n)
    target = hs.lights[light, 12:15]
    d = target - origin
    dist = np.linalg.norm(d, axis=1)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = origin
    rays[:, 3] = 1e-3
    rays[:, 4:7] = d / dist[:, None]
    rays[:, 7] = dist - 1e-3
    scene = rlm.Scene.from_host_scene(ctx, hs)
    hits = torch.zeros(n, dtype=torch.int32, device="cuda")
    rlm.trace_shadow(ctx, scene, torch.from_numpy(rays).cuda(), hits)
    ctx.check()
    scene.close()
    got = hits.cpu().numpy().astype(np.uint32)
    lib = oracle.load()
    lib.oracle_f32_any_hit_omp.argtypes = [ctypes.POINTER(oracle.Scene), ctypes.c_void_p, ctypes.c_uint32,
                                           ctypes.c_void_p]
    osc = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants,
                             oracle.triangles_v0e1e2(hs.triangles))
    want = np.zeros(n, np.uint32)
    lib.oracle_f32_any_hit_omp(ctypes.byref(osc.struct), rays.ctypes.data, n, want.ctypes.data)
    assert 0.05 < want.mean() < 0.95
    assert np.array_equal(got, want)
