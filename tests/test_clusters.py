"""Light clustering (risltc_cluster_lights): a deterministic k-means partition."""
import numpy as np


def test_kmeans_partition_is_a_fixed_point_and_deterministic():
    from risltc_gb300 import scenes
    hs = scenes.plane_of_quads(16, 16, light_count=600, seed=4)
    c1, off1 = scenes.cluster_lights(hs, 32, seed=9)
    c2, off2 = scenes.cluster_lights(hs, 32, seed=9)
    assert np.array_equal(off1, off2) and np.array_equal(c1.lights, c2.lights)
    assert off1[0] == 0 and off1[-1] == 600 and np.all(np.diff(off1.astype(np.int64)) >= 0)
    # Every light appears once.
    rows = {r.tobytes() for r in hs.lights}
    assert {r.tobytes() for r in c1.lights} == rows and len(rows) == 600
    # Each light is nearest to its own cluster's mean (Lloyd converged).
    centers = scenes.light_centers(c1.lights).astype(np.float64)
    sizes = np.diff(off1.astype(np.int64))
    label = np.repeat(np.arange(32), sizes)
    means = np.stack([centers[label == c].mean(0) if sizes[c] else np.full(3, np.inf) for c in range(32)])
    d = ((centers[:, None, :] - means[None, :, :]) ** 2).sum(-1)
    own = d[np.arange(600), label]
    assert np.all(own <= d.min(1) * (1 + 1e-9) + 1e-12)
    assert (sizes > 0).sum() >= 30
