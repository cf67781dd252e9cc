"""The GPU heightfield G-buffer producer (risltc_gbuffer_heightfield) against
the NumPy restatement of the same surface and camera (scenes.heightfield)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_heightfield_gbuffer_matches_numpy(gpu):
    import torch
    import risltc_gb300 as rl
    w, h = 240, 135
    hs = rl.scenes.heightfield(w, h, light_count=8, triangle_count=0, seed=4)
    ctx = rl.Context(0)
    planes, prim = rl.scenes.heightfield_gbuffer_gpu(ctx, w, h, seed=4)
    ctx.check()
    torch.cuda.synchronize()
    g = planes.cpu().numpy()
    p = prim.cpu().numpy().view(np.uint32)
    ctx.close()
    hit_np = hs.primitive == 0
    hit = p == 0
    assert (hit == hit_np).mean() > 0.999
    both = hit & hit_np
    assert both.sum() > 0.5 * w * h
    pos = np.abs(g[0:3, both] - hs.gbuffer[0:3, both])
    assert np.quantile(pos, 0.999) < 2e-3 and pos.max() < 5e-2
    for lo, hi in ((3, 6), (6, 9)):
        dots = (g[lo:hi, both] * hs.gbuffer[lo:hi, both]).sum(0)
        assert np.quantile(dots, 0.001) > 0.9999
    assert np.abs(g[9, both] - hs.gbuffer[9, both]).max() < 1e-2
    # Materials: ranges and means of the hashed uniforms.
    rough, albedo = g[16, both], g[10:13, both]
    assert rough.min() >= 0.05 and rough.max() <= 1.0 and abs(rough.mean() - 0.525) < 0.01
    assert albedo.min() >= 0.2 and albedo.max() <= 0.8 and abs(albedo.mean() - 0.5) < 0.01
    assert np.all(g[13:16, both] == np.float32(0.02))
