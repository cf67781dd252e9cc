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
