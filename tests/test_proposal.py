"""The cluster proposal of the RIS candidates (risltc_proposal_clusters).

CPU: the oracle's proposal draws lights with exactly the probabilities it
reports.  GPU: the CUDA path equals the oracle bit for bit (candidates,
reservoirs, pixels), and the estimate stays unbiased: against the reference's
ground-truth estimator (uniform light choice, PSA sampling) the per-pixel
z-scores over 4096 spp are standard normal.
"""
import ctypes

import numpy as np
import pytest

import golden_data as gd
import oracle


def clustered(sc, k, seed=3):
    from risltc_gb300 import scenes
    order, offsets = scenes.cluster_order(sc["lights"], k, seed)
    lights = np.ascontiguousarray(sc["lights"][order])
    bounds, power = scenes.cluster_summaries(lights, sc["max_vertex_count"], offsets)
    return dict(sc, lights=lights), offsets, bounds, power


def oracle_scene(sc, offsets, bounds, power, shadows=True):
    tris = oracle.triangles_v0e1e2(sc["triangles"]) if shadows and len(sc["triangles"]) else None
    l0, l1, k = gd.ltc()
    osc = oracle.OracleScene(sc["lights"], sc["max_vertex_count"], l0, l1, k, tris)
    osc.set_clusters(offsets, bounds, power)
    return osc


def test_oracle_proposal_draws_its_reported_probabilities():
    sc, offsets, bounds, power = clustered(gd.scene("quads"), 16)
    osc = oracle_scene(sc, offsets, bounds, power)
    lib = oracle.load()
    lib.oracle_f32_proposal.argtypes = [ctypes.POINTER(oracle.Scene), ctypes.POINTER(oracle.Settings)] + \
        [ctypes.c_void_p] * 2 + [ctypes.c_uint32] * 3 + [ctypes.c_void_p] * 2
    n_lights = sc["lights"].shape[0]
    sizes = np.diff(offsets.astype(np.int64))
    g = sc["gbuffer"]
    for pixel in (5, 300, 777):
        x = np.ascontiguousarray(g[0:3, pixel], np.float32)
        nrm = np.ascontiguousarray(g[3:6, pixel], np.float32)
        lights, pdfs = [], []
        for rn in range(8):
            st = oracle.make_settings(candidates=4096, proposal=True, proposal_uniform_fraction=0.1,
                                      random_number_proposal=0x9000 + 77 * rn)
            li = np.zeros(4096, np.int32)
            pd = np.zeros(4096, np.float32)
            lib.oracle_f32_proposal(ctypes.byref(osc.struct), ctypes.byref(st), x.ctypes.data, nrm.ctypes.data,
                                    pixel % sc["width"], pixel // sc["width"], sc["width"], li.ctypes.data,
                                    pd.ctypes.data)
            lights.append(li)
            pdfs.append(pd)
        lights, pdfs = np.concatenate(lights), np.concatenate(pdfs)
        assert lights.min() >= 0 and lights.max() < n_lights and np.all(pdfs > 0)
        # One probability per light, and they sum to one.
        per_light = np.zeros(n_lights)
        for l in np.unique(lights):
            vals = np.unique(pdfs[lights == l])
            assert vals.size == 1
            per_light[l] = vals[0]
        assert np.all(per_light > 0)
        assert abs(per_light.sum() - 1.0) < 1e-5
        # Cluster frequencies follow the probabilities (chi-square).
        cluster = np.repeat(np.arange(16), sizes)
        expected = np.bincount(cluster, weights=per_light, minlength=16) * lights.size
        observed = np.bincount(cluster[lights], minlength=16)
        chi2 = ((observed - expected) ** 2 / expected).sum()
        assert chi2 < 15 + 6 * np.sqrt(30)


@pytest.fixture(scope="module")
def rl(gpu):
    import torch
    import risltc_gb300 as rl
    ctx = rl.Context(0)
    yield rl, ctx, torch
    ctx.close()


def gpu_scene(rl_tuple, sc, offsets):
    rl, ctx, torch = rl_tuple
    l0, l1, k = gd.ltc()
    scene = rl.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    scene.set_clusters(offsets)
    return scene


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", [("hf", 8), ("quads", 16), ("oct", 6)])
def test_proposal_kernel_matches_oracle_bit_exact(rl, name, k):
    rlm, ctx, torch = rl
    sc, offsets, bounds, power = clustered(gd.scene(name), k)
    scene = gpu_scene(rl, sc, offsets)
    p = sc["width"] * sc["height"]
    out = torch.zeros((p, 3), dtype=torch.float32, device="cuda")
    res = torch.zeros((p, 4), dtype=torch.int32, device="cuda")
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    prim = None if sc["primitive"] is None else torch.from_numpy(sc["primitive"].view(np.int32)).cuda()
    frame = 2
    rlm.shade(ctx, scene, g, sc["width"], sc["height"],
              rlm.settings(candidates=16, proposal="clusters", proposal_uniform_fraction=0.2), noise_seed=frame,
              out_rgb=out, reservoirs=res, primitive=prim)
    ctx.check()
    scene.close()
    rn = rlm.noise_constants(frame)
    st = oracle.make_settings(candidates=16, proposal=True, proposal_uniform_fraction=0.2,
                              random_number_proposal=rn[1])
    orgb, ores, _ = oracle.render(oracle_scene(sc, offsets, bounds, power), st, sc["gbuffer"], sc["width"],
                                  sc["height"], rn[0], primitive=sc["primitive"], threads=0)
    r = res.cpu().numpy()
    assert np.array_equal(r[:, 0], ores["light_index"])
    assert np.array_equal(r[:, 1:3].copy().view(np.float32)[:, 0], ores["w_sum"].astype(np.float32))
    assert np.array_equal(out.cpu().numpy(), orgb)


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", [("hf", 8), ("oct", 6)])
def test_proposal_estimate_is_unbiased(rl, name, k):
    from test_unbiased import BATCHES, FRAMES_PER_BATCH
    rlm, ctx, torch = rl
    sc, offsets, _, _ = clustered(gd.scene(name), k)
    scene = gpu_scene(rl, sc, offsets)
    p = sc["width"] * sc["height"]
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    prim = None if sc["primitive"] is None else torch.from_numpy(sc["primitive"].view(np.int32)).cuda()
    out = torch.zeros((p, 3), dtype=torch.float32, device="cuda")

    def means(settings, seed0):
        m = np.zeros((BATCHES, p, 3))
        for b in range(BATCHES):
            rlm.shade(ctx, scene, g, sc["width"], sc["height"], settings, noise_seed=seed0 + b * FRAMES_PER_BATCH,
                      frames=FRAMES_PER_BATCH, out_rgb=out, primitive=prim)
            m[b] = out.cpu().numpy()
        return m

    a = means(rlm.settings(candidates=32, proposal="clusters", proposal_uniform_fraction=0.1), 0)
    b = means(rlm.settings(technique="projected_solid_angle", light_sampling="uniform"), 1_000_000)
    ctx.check()
    scene.close()
    ma, mb = a.mean(0), b.mean(0)
    se = np.sqrt(a.var(0, ddof=1) / BATCHES + b.var(0, ddof=1) / BATCHES)
    lit = se > 1e-6 * np.maximum(np.abs(mb), 1e-30)
    z = (ma - mb)[lit] / se[lit]
    print("%s proposal: %d pixel-channels, z mean %.3f, variance %.3f, max |z| %.2f"
          % (name, z.size, z.mean(), z.var(), np.abs(z).max()))
    assert abs(z.mean()) < 0.15
    assert 0.7 < z.var() < 1.4
    assert (np.abs(z) > 5.0).mean() < 0.002
