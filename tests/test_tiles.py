"""Tile shapes of the RIS candidate kernel and their autotuner.

Every risltc_tile_t (pixels per warp x candidates per pixel per chunk, or one
thread per pixel) evaluates the same candidates with the same operations and
replays each pixel's reservoir in candidate order, so images and reservoirs
equal the default shape's bit for bit for ragged pixel counts (not a multiple
of any tile's pixels), background pixels and candidate counts that do not
fill a chunk: every shape in exact numerics, the binned shapes in fast
numerics.  The per-pixel kernel in fast numerics has its multiply-adds
contracted differently by the compiler; it agrees within the fast-numerics
bounds of the parity tests.  risltc_autotune
and risltc_autotune_batch time every shape and keep the fastest.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(gpu):
    import torch
    import risltc_gb300 as rl
    ctx = rl.Context(0)
    hs = rl.scenes.heightfield(157, 61, 300, 4000, seed=3)
    scene = rl.Scene.from_host_scene(ctx, hs)
    g = torch.from_numpy(hs.gbuffer).cuda()
    prim = torch.from_numpy(hs.primitive.view(np.int32)).cuda()
    yield rl, torch, ctx, hs, scene, g, prim
    scene.close()
    ctx.close()


def render(env, s, frames=2, seed=11):
    rl, torch, ctx, hs, scene, g, prim = env
    out = torch.full((hs.pixels, 3), -1.0, device="cuda")
    res = torch.full((hs.pixels, 4), -7, dtype=torch.int32, device="cuda")
    rl.shade(ctx, scene, g, hs.width, hs.height, s, noise_seed=seed, frames=frames, out_rgb=out, reservoirs=res,
             primitive=prim)
    ctx.check()
    return out.cpu().numpy(), res.cpu().numpy()


@pytest.mark.parametrize("numerics", ["exact", "fast"])
# 40 and 96 candidates take two and three super-chunks per frame, so the
# binned kernels' windows of deferred items and replays (four 32-candidate
# super-chunks in exact numerics, eight 16-candidate ones in fast numerics)
# end in the middle of a frame; the per-pixel kernel evaluates each pixel's
# candidates in sequence and checks that bookkeeping independently.
@pytest.mark.parametrize("candidates", [32, 13, 8, 40, 96])
def test_every_tile_equals_the_default(env, numerics, candidates):
    rl = env[0]
    rgb0, res0 = render(env, rl.settings(candidates=candidates, numerics=numerics))
    assert np.isfinite(rgb0).all() and (res0[:, 0] >= 0).any()
    for tile in rl.api.TILES:
        rgb, res = render(env, rl.settings(candidates=candidates, numerics=numerics, tile=tile))
        if numerics == "fast" and tile == "per_pixel":
            # The fast-numerics bounds of the parity tests: the same light for
            # 99.9% of pixels, luminance within 1% at the 99th percentile.
            same = res[:, 0] == res0[:, 0]
            assert same.mean() >= 0.999
            lum, lum0 = rgb.sum(1), rgb0.sum(1)
            m = same & (lum0 > 0)
            assert np.quantile(np.abs(lum[m] - lum0[m]) / lum0[m], 0.99) <= 1e-2
            continue
        assert np.array_equal(rgb.view(np.uint32), rgb0.view(np.uint32)), tile
        assert np.array_equal(res, res0), tile


def test_tile_out_of_range_is_rejected(env):
    rl = env[0]
    s = rl.settings()
    s.tile = len(rl.api.TILES)
    with pytest.raises(rl.RisltcError):
        render(env, s)


def test_autotune_keeps_the_fastest_tile(env):
    rl, torch, ctx, hs, scene, g, prim = env
    s = rl.settings(candidates=32)
    tuned, ms = rl.autotune(ctx, scene, g, hs.width, hs.height, s, noise_seed=5, frames=1, repeats=2, primitive=prim)
    assert set(ms) == set(rl.api.TILES)
    assert all(v > 0.0 for v in ms.values())
    best = rl.api.TILE_NAMES[tuned.tile]
    assert ms[best] == min(ms.values())
    assert s.tile == rl.api.TILES["32x8"]  # the caller's settings are not touched
    assert np.array_equal(render(env, tuned)[0], render(env, s)[0])


def test_autotune_without_candidate_kernel_reports_zeros(env):
    rl, torch, ctx, hs, scene, g, prim = env
    s = rl.settings(technique="projected_solid_angle", light_sampling="uniform", tile="16x4")
    tuned, ms = rl.autotune(ctx, scene, g, hs.width, hs.height, s, repeats=1, primitive=prim)
    assert tuned.tile == rl.api.TILES["16x4"]
    assert all(v == 0.0 for v in ms.values())


def test_autotune_batch_sets_every_item_and_restores_seeds(env):
    rl, torch = env[0], env[1]
    ctx = env[2]
    hss = [rl.scenes.plane_of_quads(w, h, n, seed=40 + k, triangles=t)
           for k, (w, h, n, t) in enumerate([(64, 48, 16, 0), (97, 33, 200, 1500), (40, 40, 700, 800)])]
    scenes = [rl.Scene.from_host_scene(ctx, hs) for hs in hss]
    s = rl.settings(candidates=8)
    items = []
    for k, (hs, sc) in enumerate(zip(hss, scenes)):
        items.append(dict(scene=sc, gbuffer=torch.from_numpy(hs.gbuffer).cuda(), width=hs.width, height=hs.height,
                          settings=s, noise_seed=3 * k, frames=2,
                          out_rgb=torch.zeros((hs.pixels, 3), dtype=torch.float32, device="cuda")))
    rl.shade_batch(ctx, items)
    torch.cuda.synchronize()
    reference = [it["out_rgb"].clone() for it in items]
    # The C call leaves every item's noise seed where it was.
    arr, tables = rl.api._batch_array(items)
    ms = (ctypes.c_float * len(rl.api.TILES))()
    rl.api.check(rl._native.load().risltc_autotune_batch(ctx.handle, arr, len(items), 1, ms), "risltc_autotune_batch")
    assert [t.random_seed for t in tables] == [it["noise_seed"] for it in items]
    assert len({a.settings.tile for a in arr}) == 1
    best, ms = rl.autotune_batch(ctx, items, repeats=1)
    assert set(ms) == set(rl.api.TILES) and all(v > 0.0 for v in ms.values())
    assert ms[best] == min(ms.values())
    assert all(it["settings"].tile == rl.api.TILES[best] for it in items)
    for it in items:
        it["out_rgb"].zero_()
    seeds = rl.shade_batch(ctx, items)
    ctx.check()
    assert seeds == [3 * k + 2 for k in range(len(items))]
    for it, ref in zip(items, reference):
        assert torch.equal(it["out_rgb"], ref)
    for sc in scenes:
        sc.close()
