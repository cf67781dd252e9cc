"""NumPy restatement of the learned proposal's MLP forward pass, as the
tensor-core kernels compute it: BF16 weights, features and activations,
sums in higher precision, BF16 logits.

TEST INFRASTRUCTURE: imported only by tests/ and __graft_entry__.smoke(), as
the checker.  The product never imports it.  The model has no counterpart in
the reference; its definition (inputs, encoding, layers) is the one in
include/risltc.h (risltc_model_*).
"""
import numpy as np


def bf16(x):
    """Round FP32 to BF16 (nearest even), returned as FP32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def encode(gbuffer, center, half_extent):
    """The 144 features per pixel: for each of the 10 inputs (position centred
    and scaled, normal, outgoing direction, roughness) u, sin(2^k pi u) and
    cos(2^k pi u) for k = 0..5, then 14 zero padding features."""
    g = gbuffer.astype(np.float64)
    u = np.concatenate([(g[0:3] - np.asarray(center, np.float64)[:, None]) * np.float32(1.0 / half_extent),
                        g[3:6], g[6:9], g[16:17]], axis=0).T  # [P, 10]
    feats = []
    for i in range(10):
        x = u[:, i]
        feats += [x] + [np.sin(np.pi * x * 2.0 ** k) for k in range(6)] + [np.cos(np.pi * x * 2.0 ** k) for k in range(6)]
    f = np.stack(feats, axis=1)
    return np.concatenate([f, np.zeros((f.shape[0], 14))], axis=1).astype(np.float32)


def logits(params, k, features):
    """Forward pass from the FP32 parameter vector (W1 [64][144], b1, W2
    [64][64], b2, W3 [k][64], b3); the padding features carry no weight."""
    o = 0

    def take(n):
        nonlocal o
        v = params[o:o + n]
        o += n
        return v
    w1 = bf16(take(64 * 144)).reshape(64, 144).astype(np.float64)
    w1[:, 130:] = 0.0
    b1 = take(64).astype(np.float64)
    w2 = bf16(take(64 * 64)).reshape(64, 64).astype(np.float64)
    b2 = take(64).astype(np.float64)
    w3 = bf16(take(k * 64)).reshape(k, 64).astype(np.float64)
    b3 = take(k).astype(np.float64)
    h = bf16(features).astype(np.float64)
    h = bf16(np.maximum(h @ w1.T + b1, 0.0).astype(np.float32)).astype(np.float64)
    h = bf16(np.maximum(h @ w2.T + b2, 0.0).astype(np.float32)).astype(np.float64)
    return bf16((h @ w3.T + b3).astype(np.float32))


def _layers(params, k):
    o = 0
    out = {}
    for name, n in (("w1", 64 * 144), ("b1", 64), ("w2", 64 * 64), ("b2", 64), ("w3", k * 64), ("b3", k)):
        out[name] = np.asarray(params[o:o + n], np.float32)
        o += n
    out["w1"] = out["w1"].reshape(64, 144)
    out["w2"] = out["w2"].reshape(64, 64)
    out["w3"] = out["w3"].reshape(k, 64)
    return out


def train_gradient(params, k, features, lights, weights, light_cluster, light_count, inv_batch, valid,
                   shaded=None, chosen=None, shadowed_weight=0.5, rounding="bf16"):
    """The gradient of one training step of the learned proposal, as the
    training kernels define it (the mean over the B training pixels of the
    cross entropy between the candidates' per-cluster weight shares T and
    q = softmax(logits), plus the shadowed part: s (q - onehot(cluster of the
    chosen light)) with s = w * clamp(shaded / (sum w / M), 0, 4)), in FP64.

    features: [B, 144] encoded inputs of the training pixels; lights,
    weights: [B, M] their candidates (light index, RIS weight p_hat / p);
    light_cluster: each light's cluster; valid: [B] covered pixels; shaded,
    chosen: [B] or None.  rounding="bf16" models the tensor-core kernel (BF16
    features with feature 130 = 1 standing for layer 1's bias, BF16 weights,
    activations, logits and logit gradients, each candidate's target
    subtracted from the BF16 logit gradient in turn); "none" the FP32
    CUDA-core kernel (no rounding).  Returns the gradient vector in the
    parameter order of the model."""
    L = _layers(params, k)
    b = features.shape[0]
    m = lights.shape[1]
    r = bf16 if rounding == "bf16" else (lambda x: np.asarray(x, np.float32))
    f64 = lambda x: np.asarray(x, np.float64)  # noqa: E731
    e = np.array(features, np.float32)
    e[:, 130:] = 0.0
    w1 = np.array(L["w1"])
    w1[:, 130:] = 0.0
    w1, w2, w3 = f64(r(w1)), f64(r(L["w2"])), f64(r(L["w3"]))
    e = f64(r(e))
    h1 = f64(r(np.maximum((e @ w1.T).astype(np.float32) + L["b1"], 0.0)))
    h2 = f64(r(np.maximum((h1 @ w2.T).astype(np.float32) + L["b2"], 0.0)))
    z = f64(r((h2 @ w3.T).astype(np.float32) + L["b3"]))
    # Per-pixel target weights, summed in candidate order in FP32.
    w = np.asarray(weights, np.float32)
    total = np.zeros(b, np.float32)
    for c in range(m):
        total = (total + w[:, c]).astype(np.float32)
    learn = valid & (total > 0) & (total <= np.float32(3.0e38))
    wu = np.float32(1.0 - shadowed_weight) if shaded is not None else np.float32(1.0)
    ss = np.zeros(b, np.float32)
    if shaded is not None:
        ok = learn & (chosen >= 0)
        ratio = np.where(ok, shaded / np.where(ok, total / np.float32(m), 1), 0).astype(np.float32)
        ss = np.where(ok, np.float32(shadowed_weight) * np.clip(ratio, 0, 4), 0).astype(np.float32)
    coef = np.where(learn, (wu + ss) * np.float32(inv_batch), 0).astype(np.float64)
    q = np.exp(z - z.max(axis=1, keepdims=True))
    q /= q.sum(axis=1, keepdims=True)
    dz = r(coef[:, None] * q)
    unshadowed = np.where(learn, wu / np.where(learn, total, 1) * np.float32(inv_batch), 0).astype(np.float32)
    rows = np.arange(b)
    for c in range(m):
        lc = lights[:, c]
        ok = learn & (w[:, c] > 0) & (lc >= 0) & (lc < light_count)
        cl = light_cluster[np.where(ok, lc, 0)]
        sub = (unshadowed * w[:, c]).astype(np.float32)
        dz[rows[ok], cl[ok]] = r(dz[rows[ok], cl[ok]] - sub[ok])
    if shaded is not None:
        ok = learn & (chosen >= 0) & (chosen < light_count) & (ss > 0)
        cl = light_cluster[np.where(ok, chosen, 0)]
        sub = (ss * np.float32(inv_batch)).astype(np.float32)
        dz[rows[ok], cl[ok]] = r(dz[rows[ok], cl[ok]] - sub[ok])
    dz = f64(dz)
    d2 = f64(r((dz @ w3) * (h2 > 0)))
    d1 = f64(r((d2 @ w2) * (h1 > 0)))
    g_w1 = d1.T @ e
    g_w1[:, 130:] = 0.0
    parts = [g_w1.ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), (dz.T @ h2).ravel(), dz.sum(0)]
    return np.concatenate(parts)
