"""The converged GPU estimate is unbiased, and per-sample estimates track the
FP64 oracle.

Unbiasedness: the default estimator (RIS over all lights with the LTC-CP
target, then PSA sampling of the chosen light with MIS and shadow rays,
shading_pass.frag.glsl:723-759) and the reference's ground-truth estimator
(uniform light choice and PSA sampling, the recipe of experiment_list.c:399-407)
estimate the same integral by different means.  Both run for 4096 spp as 64
batches of 64 frames with independent noise; per pixel and channel the
difference of the two means, divided by its standard error from the batch
means, is a z-score that must look standard normal over the image.

FP64: the GPU's exact-numerics frame against the FP64 twin of the oracle (same
noise) where both choose the same light.
"""
import numpy as np
import pytest

import golden_data as gd
import oracle

pytestmark = pytest.mark.gpu

BATCHES = 64
FRAMES_PER_BATCH = 64


@pytest.fixture(scope="module")
def rl(gpu):
    import torch
    import risltc_gb300 as rl
    ctx = rl.Context(0)
    yield rl, ctx, torch
    ctx.close()


def batch_means(rl_tuple, sc, settings, seed0):
    rl, ctx, torch = rl_tuple
    l0, l1, k = gd.ltc()
    scene = rl.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    p = sc["width"] * sc["height"]
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    prim = None if sc["primitive"] is None else torch.from_numpy(sc["primitive"].view(np.int32)).cuda()
    out = torch.zeros((p, 3), dtype=torch.float32, device="cuda")
    means = np.zeros((BATCHES, p, 3), np.float64)
    for b in range(BATCHES):
        rl.shade(ctx, scene, g, sc["width"], sc["height"], settings, noise_seed=seed0 + b * FRAMES_PER_BATCH,
                 frames=FRAMES_PER_BATCH, out_rgb=out, primitive=prim)
        means[b] = out.cpu().numpy()
    ctx.check()
    scene.close()
    return means


@pytest.mark.parametrize("scene_name", ["hf", "oct"])
def test_ris_estimate_is_unbiased_against_ground_truth_estimator(rl, scene_name):
    rlm = rl[0]
    sc = gd.scene(scene_name)
    ris = rlm.settings(candidates=32)
    ground_truth = rlm.settings(technique="projected_solid_angle", light_sampling="uniform")
    a = batch_means(rl, sc, ris, 0)
    b = batch_means(rl, sc, ground_truth, 1_000_000)
    assert np.isfinite(a).all() and np.isfinite(b).all()
    ma, mb = a.mean(0), b.mean(0)
    se = np.sqrt(a.var(0, ddof=1) / BATCHES + b.var(0, ddof=1) / BATCHES)
    lit = se > 1e-6 * np.maximum(np.abs(mb), 1e-30)
    assert lit.sum() > 1000
    z = (ma - mb)[lit] / se[lit]
    print("%s: %d pixel-channels, z mean %.3f, variance %.3f, max |z| %.2f, image sums differ by %.2e"
          % (scene_name, z.size, z.mean(), z.var(), np.abs(z).max(), abs(ma.sum() - mb.sum()) / mb.sum()))
    # Standard normal over the image (1,700 to 3,900 pixel-channels).
    assert abs(z.mean()) < 0.15
    assert 0.7 < z.var() < 1.4
    assert (np.abs(z) > 5.0).mean() < 0.002
    # The two estimators agree on the image to a fraction of a percent.
    rel = np.abs(ma.sum() - mb.sum()) / mb.sum()
    assert rel < 5e-3


def test_gpu_frame_tracks_fp64_oracle(gpu):
    import risltc_gb300 as rlm
    import torch
    c = gd.config("hf_ltc_cp_m16")
    sc = gd.scene(c["scene"])
    ctx = rlm.Context(0)
    l0, l1, k = gd.ltc()
    scene = rlm.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    p = sc["width"] * sc["height"]
    out = torch.zeros((p, 3), dtype=torch.float32, device="cuda")
    res = torch.zeros((p, 4), dtype=torch.int32, device="cuda")
    frame = next(f for f in range(8) if rlm.noise_constants(f)[0] == c["random_numbers"][0])
    rlm.shade(ctx, scene, torch.from_numpy(sc["gbuffer"]).cuda(), sc["width"], sc["height"],
              rlm.settings(candidates=c["candidates"]), noise_seed=frame, out_rgb=out, reservoirs=res,
              primitive=None if sc["primitive"] is None else torch.from_numpy(sc["primitive"].view(np.int32)).cuda())
    ctx.check()
    rgb, light = out.cpu().numpy(), res.cpu().numpy()[:, 0]
    scene.close()
    ctx.close()
    tris = oracle.triangles_v0e1e2(sc["triangles"]) if len(sc["triangles"]) else None
    osc = oracle.OracleScene(sc["lights"], sc["max_vertex_count"], l0, l1, k, tris)
    st = oracle.make_settings(candidates=c["candidates"])
    rgb64, res64, _ = oracle.render(osc, st, sc["gbuffer"], sc["width"], sc["height"], c["random_numbers"][0],
                                    primitive=sc["primitive"], precision="f64")
    same = (light == res64["light_index"]) & (light >= 0)
    assert same.mean() > 0.95
    rel = np.abs(rgb[same] - rgb64[same]) / np.maximum(np.abs(rgb64[same]), 1e-6)
    # The FP32 path's own distance from FP64 (the GPU is bit-identical to the
    # FP32 oracle): typical pixels agree to about 1e-6; the tail comes from
    # the cancellation of the LTC edge sums of small, distant polygons, which
    # enters the estimate through the reservoir weight w_sum / (M p_hat).
    print("GPU vs FP64 oracle, relative error: median %.2e, 99%% %.2e, max %.2e"
          % (np.median(rel), np.quantile(rel, 0.99), rel.max()))
    assert np.median(rel) < 1e-5
    assert np.quantile(rel, 0.99) < 5e-3
