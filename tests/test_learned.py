"""The learned cluster proposal's model (risltc_model_*): the tensor-core
forward pass against a NumPy restatement (BF16 weights and activations, FP32
sums), and the learned proposal's unbiasedness."""
import numpy as np
import pytest

import golden_data as gd
import mlp_numpy
from test_proposal import clustered

bf16 = mlp_numpy.bf16
encode = mlp_numpy.encode
reference_logits = mlp_numpy.logits


def test_parameter_count():
    import risltc_gb300 as rl
    lib = rl._native.load()
    assert lib.risltc_model_parameter_count(256) == 64 * 144 + 64 + 64 * 64 + 64 + 256 * 64 + 256


@pytest.mark.gpu
@pytest.mark.parametrize("k", [64, 72, 256])
def test_model_logits_match_numpy(gpu, k):
    """The tcgen05 forward pass (128-pixel tiles, clusters padded to a
    multiple of 16 and produced 128 at a time) against NumPy, on a frame
    whose pixel count is not a multiple of 128."""
    import torch
    import risltc_gb300 as rl
    sc = gd.scene("hf")
    assert (sc["width"] * sc["height"]) % 128 != 0
    ctx = rl.Context(0)
    model = rl.Model(ctx, k, seed=7)
    rng = np.random.default_rng(1)
    params = model.get_params()
    # Larger output weights and non-zero biases than the initialisation.
    params[64 * 144 + 64 + 64 * 64 + 64:] *= 10.0
    params[64 * 144:64 * 144 + 64] = rng.normal(0, 0.1, 64)
    model.set_params(params)
    center, half = (0.5, -0.25, 1.0), 6.0
    model.set_input_transform(center, half)
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    got = model.logits(g, sc["width"], sc["height"]).cpu().numpy()
    ctx.check()
    model.close()
    ctx.close()
    want = reference_logits(params, k, encode(sc["gbuffer"], center, half))
    err = np.abs(got - want)
    scale = np.abs(want).max()
    # The restatement rounds to BF16 where the kernel does; they differ only
    # where an FP32 sum in another order lands on the other side of a BF16
    # rounding boundary (one BF16 step is 2^-8 relative; measured largest
    # difference 0.23% of the largest logit, median 0).
    assert np.quantile(err, 0.999) <= 0.005 * scale
    assert err.max() <= 0.01 * scale
    print("logits: scale %.3f, median error %.2e, max error %.2e" % (scale, np.median(err), err.max()))


@pytest.mark.gpu
def test_learned_proposal_is_unbiased(gpu):
    import torch
    import risltc_gb300 as rl
    from test_unbiased import BATCHES, FRAMES_PER_BATCH
    sc, offsets, _, _ = clustered(gd.scene("hf"), 8)
    ctx = rl.Context(0)
    l0, l1, k = gd.ltc()
    scene = rl.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    scene.set_clusters(offsets)
    model = rl.Model(ctx, 8, seed=3)
    params = model.get_params()
    params[64 * 144 + 64 + 64 * 64 + 64:] *= 20.0  # a strongly non-uniform proposal
    model.set_params(params)
    model.set_input_transform((0.0, 0.0, 1.0), 6.0)
    scene.set_model(model)
    p = sc["width"] * sc["height"]
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    out = torch.zeros((p, 3), dtype=torch.float32, device="cuda")

    def means(settings, seed0):
        m = np.zeros((BATCHES, p, 3))
        for b in range(BATCHES):
            rl.shade(ctx, scene, g, sc["width"], sc["height"], settings, noise_seed=seed0 + b * FRAMES_PER_BATCH,
                     frames=FRAMES_PER_BATCH, out_rgb=out)
            m[b] = out.cpu().numpy()
        return m

    a = means(rl.settings(candidates=32, proposal="learned", proposal_uniform_fraction=0.1), 0)
    b = means(rl.settings(technique="projected_solid_angle", light_sampling="uniform"), 1_000_000)
    ctx.check()
    scene.close()
    model.close()
    ctx.close()
    ma, mb = a.mean(0), b.mean(0)
    se = np.sqrt(a.var(0, ddof=1) / BATCHES + b.var(0, ddof=1) / BATCHES)
    lit = se > 1e-6 * np.maximum(np.abs(mb), 1e-30)
    z = (ma - mb)[lit] / se[lit]
    print("learned proposal: %d pixel-channels, z mean %.3f, variance %.3f, max |z| %.2f"
          % (z.size, z.mean(), z.var(), np.abs(z).max()))
    assert abs(z.mean()) < 0.15
    assert 0.7 < z.var() < 1.4
    assert (np.abs(z) > 5.0).mean() < 0.002


def exact_cluster_targets(sc, offsets):
    """Per pixel, each cluster's share of the LTC-CP targets of all lights
    (the distribution the learned proposal is trained towards)."""
    import ctypes
    import oracle as orc
    from test_proposal import oracle_scene
    from risltc_gb300 import scenes
    bounds, power = scenes.cluster_summaries(sc["lights"], sc["max_vertex_count"], offsets)
    osc = oracle_scene(sc, offsets, bounds, power)
    lib = orc.load()
    lib.oracle_f32_ltc_cp_targets.argtypes = [ctypes.POINTER(orc.Scene), ctypes.POINTER(orc.Settings),
                                              ctypes.POINTER(orc.GBuffer), ctypes.c_uint32, ctypes.c_void_p]
    st = orc.make_settings()
    g = orc.GBuffer()
    g.width, g.height = sc["width"], sc["height"]
    planes = np.ascontiguousarray(sc["gbuffer"], np.float32)
    g.planes = planes.ctypes.data
    n = sc["lights"].shape[0]
    k = offsets.size - 1
    cluster = np.repeat(np.arange(k), np.diff(offsets.astype(np.int64)))
    out = np.zeros((g.width * g.height, k))
    p_hat = np.zeros(n, np.float32)
    for i in range(g.width * g.height):
        lib.oracle_f32_ltc_cp_targets(ctypes.byref(osc.struct), ctypes.byref(st), ctypes.byref(g), i,
                                      p_hat.ctypes.data)
        out[i] = np.bincount(cluster, weights=p_hat.astype(np.float64), minlength=k)
    return out


def mean_kl(targets, logits):
    t = targets / np.maximum(targets.sum(1, keepdims=True), 1e-30)
    z = logits - logits.max(1, keepdims=True)
    logq = z - np.log(np.exp(z).sum(1, keepdims=True))
    keep = targets.sum(1) > 0
    kl = (t * (np.log(np.maximum(t, 1e-30)) - logq)).sum(1)
    return float(kl[keep].mean())


@pytest.mark.gpu
def test_model_logits_unaligned_frame(gpu):
    """A frame whose pixel count is not a multiple of 4: the inputs come by
    plain loads instead of bulk copies."""
    import torch
    import risltc_gb300 as rl
    sc = gd.scene("hf")
    n = sc["width"] * sc["height"] - 1
    assert n % 4 != 0
    g_host = np.ascontiguousarray(sc["gbuffer"][:, :n])
    ctx = rl.Context(0)
    model = rl.Model(ctx, 64, seed=9)
    params = model.get_params()
    center, half = (0.0, 0.0, 1.0), 6.0
    model.set_input_transform(center, half)
    got = model.logits(torch.from_numpy(g_host).cuda(), n, 1).cpu().numpy()
    ctx.check()
    model.close()
    ctx.close()
    want = reference_logits(params, 64, encode(g_host, center, half))
    err = np.abs(got - want)
    print("ragged logits: scale %.3f, max error %.2e" % (np.abs(want).max(), err.max()))
    assert err.max() <= 0.01 * np.abs(want).max()


@pytest.mark.gpu
def test_online_training_moves_the_proposal_towards_the_targets(gpu):
    import torch
    import risltc_gb300 as rl
    sc, offsets, _, _ = clustered(gd.scene("hf"), 8)
    targets = exact_cluster_targets(sc, offsets)
    ctx = rl.Context(0)
    l0, l1, k = gd.ltc()
    scene = rl.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    scene.set_clusters(offsets)
    model = rl.Model(ctx, 8, seed=5)
    model.set_input_transform((0.0, 0.0, 1.0), 6.0)
    scene.set_model(model)
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    p = sc["width"] * sc["height"]
    out = torch.zeros((p, 3), dtype=torch.float32, device="cuda")
    before = mean_kl(targets, model.logits(g, sc["width"], sc["height"]).cpu().numpy())
    model.set_training(True, learning_rate=3e-3, pixel_stride=1)
    model.set_target_mix(0.0)  # the unshadowed targets only, as computed above
    s = rl.settings(candidates=32, proposal="learned", proposal_uniform_fraction=0.1)
    for call in range(300):
        rl.shade(ctx, scene, g, sc["width"], sc["height"], s, noise_seed=call, frames=1, out_rgb=out)
    ctx.check()
    after = mean_kl(targets, model.logits(g, sc["width"], sc["height"]).cpu().numpy())
    assert np.isfinite(model.get_params()).all()
    print("KL(target || proposal): %.4f before training, %.4f after 300 steps" % (before, after))
    scene.close()
    model.close()
    ctx.close()
    assert after < 0.5 * before


@pytest.mark.gpu
def test_tensor_wait_timeout_is_reported_and_the_context_survives(gpu):
    """Fault injection on the host: the logits launch issues no tensor-core
    products, its bounded waits run out after a second, the kernel records
    the timeout and frees its tensor memory; risltc_ctx_check reports
    RISLTC_ERROR_DEVICE_TIMEOUT and the next launch is correct."""
    import torch
    import risltc_gb300 as rl
    sc = gd.scene("hf")
    ctx = rl.Context(0)
    model = rl.Model(ctx, 64, seed=3)
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    good = model.logits(g, sc["width"], sc["height"]).cpu().numpy()
    ctx.check()
    ctx.inject_fault(tensor_wait=True)
    model.logits(g, sc["width"], sc["height"])
    with pytest.raises(rl.RisltcError) as e:
        ctx.check()
    assert e.value.status == 11  # RISLTC_ERROR_DEVICE_TIMEOUT
    again = model.logits(g, sc["width"], sc["height"]).cpu().numpy()
    ctx.check()
    assert np.array_equal(again, good)
    model.close()
    ctx.close()


def gradient_blocks(k):
    """Slices of the parameter vector: W1 (real features), b1, W2, b2, W3, b3."""
    w1 = np.arange(64 * 144).reshape(64, 144)[:, :130].ravel()
    o = 64 * 144
    return [("w1", w1), ("b1", slice(o, o + 64)), ("w2", slice(o + 64, o + 64 + 4096)),
            ("b2", slice(o + 4160, o + 4224)), ("w3", slice(o + 4224, o + 4224 + 64 * k)),
            ("b3", slice(o + 4224 + 64 * k, o + 4224 + 65 * k))]


@pytest.mark.gpu
@pytest.mark.parametrize("k,candidates,stride", [(8, 32, 3), (72, 7, 7), (256, 32, 3)])
def test_tensor_core_training_gradient_matches_cuda_cores(gpu, k, candidates, stride):
    """One training step's gradient from the tcgen05 kernel (BF16 weights,
    activations and logit gradients, FP32 accumulation over the CTA's tiles)
    against the FP32 CUDA-core kernel, on the same frame and candidates with
    the shadowed target part on: each parameter block agrees within 5% of
    its largest entry and the two vectors correlate above 0.995; with
    accumulate_only the parameters do not move until apply_update.  Stride 7
    leaves a partial last tile (2,195 training pixels)."""
    import torch
    import risltc_gb300 as rl
    hs = rl.scenes.heightfield(160, 96, light_count=2048 if k > 8 else 256, triangle_count=3000, seed=11,
                               vertex_counts=(3, 8))
    order, offsets = rl.scenes.cluster_order(hs.lights, k, 3)
    lights = np.ascontiguousarray(hs.lights[order])
    ctx = rl.Context(0)
    l0, l1, kk = gd.ltc()
    scene = rl.Scene(ctx, lights, hs.max_vertex_count, l0, l1, kk, hs.triangles)
    scene.set_clusters(offsets)
    model = rl.Model(ctx, k, seed=5)
    params = model.get_params()
    params[64 * 144 + 64 + 64 * 64 + 64:] *= 10.0  # a non-uniform proposal
    model.set_params(params)
    model.set_input_transform((0.0, 0.0, 1.0), 6.0)
    scene.set_model(model)
    model.set_training(True, learning_rate=1e-3, pixel_stride=stride)
    model.set_target_mix(0.5)
    g = torch.from_numpy(np.ascontiguousarray(hs.gbuffer)).cuda()
    prim = torch.from_numpy(np.ascontiguousarray(hs.primitive).view(np.int32)).cuda()
    out = torch.zeros((hs.width * hs.height, 3), dtype=torch.float32, device="cuda")
    s = rl.settings(candidates=candidates, proposal="learned", proposal_uniform_fraction=0.1)
    grads = []
    for cuda_cores in (False, True):
        model.set_training_flags(cuda_cores=cuda_cores, accumulate_only=True)
        rl.shade(ctx, scene, g, hs.width, hs.height, s, noise_seed=4, frames=1, out_rgb=out, primitive=prim)
        grads.append(model.get_gradient(clear=True))
    ctx.check()
    assert np.array_equal(model.get_params(), params)
    tc, ref = grads
    for name, sl in gradient_blocks(k):
        scale = np.abs(ref[sl]).max()
        err = np.abs(tc[sl] - ref[sl]).max()
        print("k=%d %s: max |g| %.3e, max error %.3e (%.2f%%)" % (k, name, scale, err, 100 * err / scale))
        assert scale > 0
        assert err <= 0.05 * scale, name
    corr = np.corrcoef(tc, ref)[0, 1]
    print("k=%d correlation %.5f" % (k, corr))
    assert corr > 0.995
    # The accumulated gradient drives one Adam step on request.
    model.set_training_flags(accumulate_only=True)
    rl.shade(ctx, scene, g, hs.width, hs.height, s, noise_seed=4, frames=1, out_rgb=out, primitive=prim)
    model.apply_update()
    moved = model.get_params()
    assert np.all(model.get_gradient() == 0.0)
    ctx.check()
    scene.close()
    model.close()
    ctx.close()
    w3 = slice(64 * 144 + 4224, 64 * 144 + 4224 + 64 * k)
    assert np.abs(moved[w3] - params[w3]).max() > 0
    assert np.array_equal(moved[:64 * 144].reshape(64, 144)[:, 130:], params[:64 * 144].reshape(64, 144)[:, 130:])


@pytest.mark.gpu
def test_training_tensor_wait_timeout_is_reported_and_the_context_survives(gpu):
    """Fault injection on the host for the tensor-core training kernel: it
    issues no products, its bounded waits run out, it records the timeout,
    adds nothing to the gradient and frees its tensor memory; the next
    training call works."""
    import torch
    import risltc_gb300 as rl
    sc, offsets, _, _ = clustered(gd.scene("hf"), 8)
    ctx = rl.Context(0)
    l0, l1, k = gd.ltc()
    scene = rl.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    scene.set_clusters(offsets)
    model = rl.Model(ctx, 8, seed=5)
    model.set_input_transform((0.0, 0.0, 1.0), 6.0)
    scene.set_model(model)
    model.set_training(True, learning_rate=1e-3, pixel_stride=1)
    model.set_training_flags(accumulate_only=True)
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    out = torch.zeros((sc["width"] * sc["height"], 3), dtype=torch.float32, device="cuda")
    s = rl.settings(candidates=32, proposal="learned", proposal_uniform_fraction=0.1)
    ctx.inject_fault(train_tensor_wait=True)
    rl.shade(ctx, scene, g, sc["width"], sc["height"], s, noise_seed=2, frames=1, out_rgb=out)
    with pytest.raises(rl.RisltcError) as e:
        ctx.check()
    assert e.value.status == 11  # RISLTC_ERROR_DEVICE_TIMEOUT
    assert np.all(model.get_gradient(clear=True) == 0.0)
    rl.shade(ctx, scene, g, sc["width"], sc["height"], s, noise_seed=2, frames=1, out_rgb=out)
    ctx.check()
    assert np.abs(model.get_gradient()).max() > 0
    scene.close()
    model.close()
    ctx.close()
