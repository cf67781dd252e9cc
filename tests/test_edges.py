"""Edge cases of the shading path, through the C ABI, against the oracle.

Frames that are all background, a single pixel, a single light, one
candidate and the largest candidate count (4096) give the oracle's pixels
bit for bit in exact numerics; arguments past the limits (4097 candidates,
an empty frame) and non-finite occluders are rejected before any work.
"""
import numpy as np
import pytest

import golden_data as gd
from test_gpu_parity import gpu_render, oracle_render

pytestmark = pytest.mark.gpu

RIS = dict(technique="ltc_cp", light_sampling="ris", mis="optimal_clamped", sample_count=1, light_samples=1,
           fast_atan=False)


@pytest.fixture(scope="module")
def rl(gpu):
    import torch
    import risltc_gb300 as rl
    ctx = rl.Context(0)
    yield rl, ctx, torch
    ctx.close()


def heightfield(w, h, lights, tris, seed):
    import risltc_gb300 as rlm
    hs = rlm.scenes.heightfield(w, h, light_count=lights, triangle_count=tris, seed=seed, vertex_counts=(3, 8))
    return dict(width=hs.width, height=hs.height, gbuffer=hs.gbuffer, primitive=hs.primitive, lights=hs.lights,
                triangles=hs.triangles, max_vertex_count=hs.max_vertex_count)


def rn_of(frame):
    import risltc_gb300 as rlm
    return rlm.noise_constants(frame)[0]


def check_bit_exact(rl_tuple, sc, candidates, frame=3):
    c = dict(RIS, candidates=candidates)
    rgb, _, idx, wp = gpu_render(rl_tuple, sc, c, noise_seed=frame)
    orgb, ores, _ = oracle_render(sc, c, rn_of(frame))
    assert np.array_equal(rgb, orgb)
    assert np.array_equal(idx, ores["light_index"])
    assert np.array_equal(wp[:, 0], ores["w_sum"].astype(np.float32))
    return rgb, idx


def test_all_background_frame(rl):
    sc = heightfield(40, 24, 64, 500, seed=4)
    sc["primitive"] = np.full(sc["width"] * sc["height"], 0xFFFFFFFF, np.uint32)
    rgb, idx = check_bit_exact(rl, sc, 16)
    assert np.all(rgb == 0.0) and np.all(idx == -1)


def test_single_pixel_frame(rl):
    sc = heightfield(33, 17, 64, 500, seed=5)
    covered = np.flatnonzero(sc["primitive"] == 0)[0]
    sc["gbuffer"] = np.ascontiguousarray(sc["gbuffer"][:, covered:covered + 1])
    sc["primitive"] = sc["primitive"][covered:covered + 1].copy()
    sc["width"], sc["height"] = 1, 1
    check_bit_exact(rl, sc, 32)


def test_single_light(rl):
    sc = heightfield(48, 27, 1, 800, seed=6)
    rgb, idx = check_bit_exact(rl, sc, 8)
    lit = idx >= 0
    assert lit.any() and np.all(idx[lit] == 0)


@pytest.mark.parametrize("candidates", [1, 4096])
def test_candidate_count_limits(rl, candidates):
    sc = heightfield(16, 8, 300, 800, seed=7)
    check_bit_exact(rl, sc, candidates)


def test_arguments_past_the_limits_are_rejected(rl):
    rlm, ctx, torch = rl
    sc = heightfield(16, 8, 16, 100, seed=8)
    l0, l1, k = gd.ltc()
    scene = rlm.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    g = torch.from_numpy(sc["gbuffer"]).cuda()
    out = torch.full((sc["width"] * sc["height"], 3), -1.0, device="cuda")
    with pytest.raises(rlm.RisltcError):
        rlm.shade(ctx, scene, g, sc["width"], sc["height"], rlm.settings(candidates=4097), out_rgb=out)
    with pytest.raises(rlm.RisltcError):
        rlm.shade(ctx, scene, g, 0, sc["height"], rlm.settings(), out_rgb=out)
    with pytest.raises(rlm.RisltcError):
        rlm.shade(ctx, scene, g, sc["width"], sc["height"], rlm.settings(), frames=0, out_rgb=out)
    ctx.check()
    assert torch.all(out == -1.0)  # nothing ran
    scene.close()
    bad = sc["triangles"].copy()
    bad[3, 4] = np.nan
    with pytest.raises(rlm.RisltcError):
        rlm.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, bad)


def test_closing_the_context_first_destroys_its_scenes_and_models(rl):
    """Closing a context destroys the scenes and models made on it first, so
    their own close (or finalizer, in any order at interpreter exit) never
    reaches a destroyed context."""
    rlm, _, torch = rl
    ctx = rlm.Context(0)
    sc = heightfield(16, 8, 16, 100, seed=9)
    l0, l1, k = gd.ltc()
    scene = rlm.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    model = rlm.Model(ctx, 8, seed=1)
    ctx.close()
    assert not scene.handle and not model.handle
    scene.close()
    model.close()
    del scene, model, ctx


def test_large_lights_close_to_the_surface(rl):
    """Large triangles and quads just above the surface: seen from the pixels
    below them, consecutive vertices lie 90 degrees or more apart and many
    polygons straddle the horizon, so the candidate kernel's branch-free
    first pass defers these items, and the deferred items' own branch-free
    pass falls back to the general path.  Bit for bit the oracle's frame."""
    import risltc_gb300 as rlm
    sc = heightfield(48, 27, 4, 600, seed=12)
    covered = sc["primitive"] == 0
    pos = sc["gbuffer"][0:3].T[covered].astype(np.float64)
    top = float(pos[:, 2].max()) + 0.05
    rng = np.random.default_rng(13)
    specs = []
    for k in range(24):
        n = 3 + k % 3
        ang = 2.0 * np.pi * np.arange(n) / n + rng.uniform(0.0, 2.0 * np.pi)
        verts = np.stack([np.cos(ang), np.sin(ang)], axis=1)
        c = pos[rng.integers(len(pos))]
        specs.append(rlm.scenes.LightSpec((np.pi + rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2), 0.0),
                                          (rng.uniform(1.5, 3.0),) * 2, (c[0], c[1], top + rng.uniform(0.0, 0.1)),
                                          tuple(np.exp(rng.uniform(np.log(0.5), np.log(5.0), 3))), verts))
    sc["lights"], sc["max_vertex_count"] = rlm.scenes.build_lights(specs)
    # The geometry does what the test is for: some pixel sees two consecutive
    # vertices of some light 90 degrees or more apart.
    nv = sc["lights"][:, 8].view(np.uint32)
    world = sc["lights"][:, 12:].reshape(len(specs), -1, 4)[:, :, :3].astype(np.float64)
    obtuse = False
    for li in range(len(specs)):
        d = world[li, :nv[li]][None, :, :] - pos[:, None, :]
        d /= np.linalg.norm(d, axis=2, keepdims=True)
        obtuse |= bool((np.sum(d * np.roll(d, -1, axis=1), axis=2) <= 0.0).any())
    assert obtuse
    check_bit_exact(rl, sc, 32)


def test_ray_count_of_the_last_call(rl):
    """risltc_ctx_ray_count reports the shadow rays the last call traced
    through its ray queue: at most two per covered pixel-frame, the same for
    the same noise, none without shadows."""
    rlm, ctx, torch = rl
    sc = heightfield(64, 36, 48, 800, seed=14)
    l0, l1, k = gd.ltc()
    scene = rlm.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    g = torch.from_numpy(sc["gbuffer"]).cuda()
    prim = torch.from_numpy(sc["primitive"].view(np.int32)).cuda()
    out = torch.zeros((sc["width"] * sc["height"], 3), device="cuda")
    counts = []
    for shadows in (True, True, False):
        rlm.shade(ctx, scene, g, sc["width"], sc["height"], rlm.settings(candidates=8, shadows=shadows),
                  noise_seed=5, frames=2, out_rgb=out, primitive=prim)
        counts.append(ctx.ray_count())
    ctx.check()
    scene.close()
    covered = int((sc["primitive"] == 0).sum())
    assert 0 < counts[0] <= 2 * 2 * covered
    assert counts[1] == counts[0]
    assert counts[2] == 0
