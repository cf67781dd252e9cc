"""Known-answer tests of the oracle's sampling routines and the multi-rank
row partition (CPU; two gloo ranks)."""
import ctypes
import os

import numpy as np
import pytest

import oracle


def psa(verts, rnd):
    lib = oracle.load()
    lib.oracle_f32_psa_sample.restype = ctypes.c_float
    lib.oracle_f32_psa_sample.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
    v = np.ascontiguousarray(verts, np.float32)
    r = np.ascontiguousarray(rnd, np.float32)
    dirs = np.zeros((len(r), 3), np.float32)
    err = np.zeros(len(r), np.float32)
    total = lib.oracle_f32_psa_sample(len(v), v.ctypes.data, len(r), r.ctypes.data, dirs.ctypes.data, err.ctypes.data)
    return total, dirs, err


def ltc_integral(verts):
    lib = oracle.load()
    lib.oracle_f32_calculate_ltc.restype = ctypes.c_float
    lib.oracle_f32_calculate_ltc.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
    v = np.ascontiguousarray(verts, np.float32)
    return lib.oracle_f32_calculate_ltc(len(v), v.ctypes.data)


def lambert_psa(verts):
    """Projected solid angle of a polygon above z = 0 (Lambert's formula, FP64)."""
    v = np.asarray(verts, np.float64)
    v = v / np.linalg.norm(v, axis=1, keepdims=True)
    total = 0.0
    for i in range(len(v)):
        a, b = v[i], v[(i + 1) % len(v)]
        c = np.cross(a, b)
        total += np.arccos(np.clip(a @ b, -1, 1)) * c[2] / np.linalg.norm(c)
    return 0.5 * abs(total)


def polygon(n, center, radius, rng):
    ang = np.sort(rng.uniform(0, 2 * np.pi, n))
    p = np.stack([center[0] + radius * np.cos(ang), center[1] + radius * np.sin(ang), np.full(n, center[2])], 1)
    return p  # counter-clockwise from above: clockwise as seen from the origin


def test_psa_of_huge_polygon_is_pi():
    sq = np.array([[-1e3, -1e3, 1.0], [1e3, -1e3, 1.0], [1e3, 1e3, 1.0], [-1e3, 1e3, 1.0]])
    total, _, _ = psa(sq, np.zeros((1, 2)))
    assert abs(total - np.pi) < 1e-5 * np.pi


@pytest.mark.parametrize("seed", range(6))
def test_psa_and_ltc_integral_agree_with_lambert(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(3, 9))
    center = (rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(0.3, 2.0))
    v = polygon(n, center, rng.uniform(0.2, 1.5), rng)
    exact = lambert_psa(v)
    total, _, _ = psa(v, np.zeros((1, 2)))
    assert abs(total - exact) <= 2e-5 * exact + 1e-7
    # calculate_ltc is the form factor PSA / pi: its rational fit
    # (polygon_sampling.glsl:514-518) approximates theta / (2 pi sin(theta)).
    assert abs(np.pi * ltc_integral(v) - exact) <= 2e-3 * exact + 1e-6


@pytest.mark.parametrize("seed", range(4))
def test_psa_samples_are_cosine_distributed(seed):
    rng = np.random.default_rng(100 + seed)
    v = polygon(int(rng.integers(3, 8)), (rng.uniform(-1.5, 1.5), rng.uniform(-1.5, 1.5), 1.0), 0.8, rng)
    n = 200_000
    total, dirs, err = psa(v, rng.random((n, 2)))
    assert np.all(dirs[:, 2] > 0)
    # E[x] under p = cos/PSA equals (1/PSA) * int x cos domega: quadrature on the polygon plane.
    pts = rng.random((400_000, 2))
    tri = []
    for i in range(1, len(v) - 1):
        a, b, c = v[0], v[i], v[i + 1]
        area = 0.5 * np.linalg.norm(np.cross(b - a, c - a))
        tri.append((a, b, c, area))
    areas = np.array([t[3] for t in tri])
    pick = rng.choice(len(tri), size=len(pts), p=areas / areas.sum())
    u, w = pts[:, 0], pts[:, 1]
    flip = u + w > 1
    u[flip], w[flip] = 1 - u[flip], 1 - w[flip]
    A = np.array([tri[k][0] for k in pick])
    B = np.array([tri[k][1] for k in pick])
    C = np.array([tri[k][2] for k in pick])
    p = A + u[:, None] * (B - A) + w[:, None] * (C - A)
    r = np.linalg.norm(p, axis=1)
    weight = (p[:, 2] / r) * p[:, 2] / r ** 3  # cos(theta) * (cos at light / r^2)
    integral_x = areas.sum() * np.mean((p[:, 0] / r) * weight)
    integral_1 = areas.sum() * np.mean(weight)
    assert abs(integral_1 - total) < 0.01 * total
    mean_x = dirs[:, 0].mean()
    se = dirs[:, 0].std() / np.sqrt(n)
    assert abs(mean_x - integral_x / integral_1) < 5 * se + 2e-3
    # Two refinement iterations leave practically no backward error.
    assert np.quantile(np.abs(err), 0.999) < 1e-4


def test_row_bands_cover_the_frame():
    from risltc_gb300.sharding import row_band
    for world in (1, 2, 3, 8):
        for h in (1, 7, 1080):
            bands = [row_band(r, world, h) for r in range(world)]
            assert bands[0][0] == 0 and bands[-1][1] == h
            assert all(bands[i][1] == bands[i + 1][0] for i in range(world - 1))
    with pytest.raises(ValueError):
        row_band(2, 2, 10)


def _shard_worker(rank, world, port, out_dir):
    import torch.distributed as dist
    import golden_data as gd
    from risltc_gb300.sharding import row_band
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    c = gd.config("hf_ltc_cp_m16")
    sc = gd.scene(c["scene"])
    l0, l1, k = gd.ltc()
    osc = oracle.OracleScene(sc["lights"], sc["max_vertex_count"], l0, l1, k, oracle.triangles_v0e1e2(sc["triangles"]))
    st = oracle.make_settings(candidates=c["candidates"])
    b0, b1 = row_band(rank, world, sc["height"])
    rgb, _, _ = oracle.render(osc, st, sc["gbuffer"], sc["width"], sc["height"], c["random_numbers"][0],
                              primitive=sc["primitive"], rows=(b0, b1), threads=1, reservoirs=False)
    band = torch.from_numpy(rgb[b0 * sc["width"]:b1 * sc["width"]].copy())
    sizes = [None] * world
    dist.all_gather_object(sizes, band.shape[0])
    gathered = [torch.zeros((s, 3)) for s in sizes]
    dist.all_gather(gathered, band) if len(set(sizes)) == 1 else [
        dist.broadcast(g.copy_(band) if r == rank else g, src=r) for r, g in enumerate(gathered)]
    if rank == 0:
        np.save(os.path.join(out_dir, "frame.npy"), torch.cat(gathered).numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_row_sharding_reproduces_single_frame(tmp_path):
    import socket
    import torch.multiprocessing as mp
    import golden_data as gd
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_shard_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    frame = np.load(tmp_path / "frame.npy")
    c = gd.config("hf_ltc_cp_m16")
    sc = gd.scene(c["scene"])
    l0, l1, k = gd.ltc()
    osc = oracle.OracleScene(sc["lights"], sc["max_vertex_count"], l0, l1, k, oracle.triangles_v0e1e2(sc["triangles"]))
    whole, _, _ = oracle.render(osc, oracle.make_settings(candidates=c["candidates"]), sc["gbuffer"], sc["width"],
                                sc["height"], c["random_numbers"][0], primitive=sc["primitive"])
    assert np.array_equal(frame, whole)
