"""The learned proposal's training step against an independent oracle.

risltc_model_train runs one training step on caller-supplied RIS candidates
(light, weight p_hat / p), the step risltc_shade takes after a frame with
training on.  Its gradient (accumulated without an Adam step) is compared
with oracle/mlp_numpy.train_gradient, an FP64 NumPy restatement of the loss's
gradient (checked against finite differences of the loss on the CPU below):
the FP32 CUDA-core kernel against the unrounded gradient, the tcgen05 kernel
against the same gradient with the kernel's BF16 roundings (features,
weights, activations, logits and logit gradients).  Cases: 8, 72 and 256
clusters (all weight gradients in tensor memory), 520 and 1024 clusters (the
output layer in chunks of 128, a partial last chunk at 520), an odd candidate count, invalid and zero-weight candidates,
background pixels, a training stride that leaves a partial last 128-pixel
tile, with and without the shadowed target part.  The training signal
replaces the reference's uniform candidate pdf p = 1/N
(shading_pass.frag.glsl:730-734).
"""
import numpy as np
import pytest

import mlp_numpy

# Largest error per parameter block, relative to the block's largest entry.
FP32_KERNEL_TOLERANCE = 1e-3    # FP32 CUDA cores, FP32 atomics over the pixels, against FP64
TENSOR_KERNEL_TOLERANCE = 2e-2  # BF16 operands modelled; FP32 accumulation order and exp differ


def blocks(k):
    o = 64 * 144
    return [("w1", slice(0, o)), ("b1", slice(o, o + 64)), ("w2", slice(o + 64, o + 4160)),
            ("b2", slice(o + 4160, o + 4224)), ("w3", slice(o + 4224, o + 4224 + 64 * k)),
            ("b3", slice(o + 4224 + 64 * k, o + 4224 + 65 * k))]


def test_oracle_gradient_equals_finite_differences():
    """The unrounded oracle is the derivative of the mean cross entropy
    between the candidates' cluster shares and softmax(logits)."""
    rng = np.random.default_rng(0)
    k, b, m, n_lights = 8, 40, 5, 30
    count = 64 * 144 + 64 + 64 * 64 + 64 + 65 * k
    params = rng.normal(0, 0.1, count).astype(np.float32)
    f = rng.normal(size=(b, 144)).astype(np.float32)
    lights = rng.integers(0, n_lights, (b, m))
    w = rng.uniform(0, 1, (b, m)).astype(np.float32)
    cluster = rng.integers(0, k, n_lights)
    g = mlp_numpy.train_gradient(params, k, f, lights, w, cluster, n_lights, 1.0 / b, np.ones(b, bool),
                                 rounding="none")

    def loss(p):
        L = mlp_numpy._layers(p, k)
        e = f.astype(np.float64)
        e[:, 130:] = 0
        w1 = L["w1"].astype(np.float64).copy()
        w1[:, 130:] = 0
        h1 = np.maximum(e @ w1.T + L["b1"], 0)
        h2 = np.maximum(h1 @ L["w2"].T + L["b2"], 0)
        z = h2 @ L["w3"].T + L["b3"]
        z = z - z.max(1, keepdims=True)
        logq = z - np.log(np.exp(z).sum(1, keepdims=True))
        t = np.zeros((b, k))
        for c in range(m):
            np.add.at(t, (np.arange(b), cluster[lights[:, c]]), w[:, c])
        t /= t.sum(1, keepdims=True)
        return -(t * logq).sum() / b

    p64 = params.astype(np.float64)
    for j in rng.choice(count, 24, replace=False):
        h = 1e-4
        a, c = p64.copy(), p64.copy()
        a[j] += h
        c[j] -= h
        fd = (loss(a) - loss(c)) / (2 * h)
        assert abs(fd - g[j]) <= 1e-3 * max(abs(fd), 1e-4), j


@pytest.fixture(scope="module")
def setup(gpu):
    import torch
    import risltc_gb300 as rl
    hs0 = rl.scenes.heightfield(150, 90, light_count=2400, triangle_count=0, seed=9, vertex_counts=(3, 8))
    ctx = rl.Context(0)
    yield rl, torch, ctx, hs0
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("k,m,stride,phase,shadowed", [(8, 13, 3, 1, True), (72, 7, 5, 2, False),
                                                       (256, 32, 3, 0, True), (520, 11, 3, 1, True),
                                                       (1024, 32, 2, 0, False)])
def test_training_gradient_matches_oracle(setup, k, m, stride, phase, shadowed):
    rl, torch, ctx, hs0 = setup
    hs, offsets = rl.scenes.cluster_lights(hs0, k, seed=3)
    n_lights = hs.light_count
    light_cluster = np.repeat(np.arange(k), np.diff(offsets.astype(np.int64)))
    scene = rl.Scene.from_host_scene(ctx, hs)
    scene.set_clusters(offsets)
    model = rl.Model(ctx, k, seed=5)
    params = model.get_params()
    rng = np.random.default_rng(k)
    params[64 * 144 + 64 + 64 * 64 + 64:] *= 10.0  # a non-uniform proposal
    params[64 * 144:64 * 144 + 64] = rng.normal(0, 0.05, 64)
    model.set_params(params)
    center, half = (0.0, 0.0, 1.0), 6.0
    model.set_input_transform(center, half)
    scene.set_model(model)
    model.set_target_mix(0.5)
    p = hs.pixels
    # Candidates of every pixel: random lights with log-uniform weights, a few
    # of weight 0 and a few naming no light.
    lights = rng.integers(0, n_lights, (p, m)).astype(np.int32)
    weights = np.exp(rng.uniform(np.log(1e-3), np.log(10.0), (p, m))).astype(np.float32)
    weights[rng.uniform(size=(p, m)) < 0.05] = 0.0
    lights[rng.uniform(size=(p, m)) < 0.01] = -1
    lights[rng.uniform(size=(p, m)) < 0.01] = n_lights + 3
    cand = np.zeros((p, m, 2), np.int32)
    cand[:, :, 0] = lights
    cand[:, :, 1] = weights.view(np.int32)
    shaded = rng.uniform(0.0, 3.0, p).astype(np.float32)
    chosen = rng.integers(-1, n_lights, p).astype(np.int32)
    res = np.zeros((p, 4), np.int32)
    res[:, 0] = chosen
    # Some background pixels, which the step must skip.
    primitive = hs.primitive.copy()
    primitive[::11] = 0xFFFFFFFF
    g = torch.from_numpy(hs.gbuffer).cuda()
    prim = torch.from_numpy(primitive.view(np.int32)).cuda()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    d_cand, d_shaded, d_res = dev(cand), dev(shaded), dev(res)
    grads = {}
    for cuda_cores in (True, False):
        model.set_training_flags(cuda_cores=cuda_cores, accumulate_only=True)
        model.train(scene, g, hs.width, hs.height, d_cand, stride, phase, d_shaded if shadowed else None,
                    d_res if shadowed else None, primitive=prim)
        grads[cuda_cores] = model.get_gradient(clear=True)
    ctx.check()
    assert np.array_equal(model.get_params(), params)
    scene.close()
    model.close()
    train = np.arange(phase, p, stride)
    inv_batch = np.float32(1.0) / np.float32(train.size)
    valid = primitive[train] != 0xFFFFFFFF
    assert (~valid).any() and valid.any()
    feats = mlp_numpy.encode(hs.gbuffer[:, train], center, half)
    args = (params, k, feats, lights[train], weights[train], light_cluster, n_lights, inv_batch, valid)
    extra = dict(shaded=shaded[train], chosen=chosen[train], shadowed_weight=0.5) if shadowed else {}
    for cuda_cores, rounding, tol in ((True, "none", FP32_KERNEL_TOLERANCE), (False, "bf16", TENSOR_KERNEL_TOLERANCE)):
        want = mlp_numpy.train_gradient(*args, rounding=rounding, **extra)
        got = grads[cuda_cores]
        for name, sl in blocks(k):
            scale = np.abs(want[sl]).max()
            err = np.abs(got[sl] - want[sl]).max()
            print("k=%d %s %s: max |g| %.3e, max error %.2e of it" % (
                k, "cuda cores" if cuda_cores else "tensor cores", name, scale, err / scale))
            assert scale > 0
            assert err <= tol * scale, (cuda_cores, name, err / scale)
