"""Seeded synthetic workloads standing in for the reference's scenes.

The reference renders the Bistro and Zero Day scenes (src/main.c:36-40); their
data directory is not distributed, so these generators produce inputs with the
shapes and value distributions of the benchmark configurations:

* plane_of_quads: a W x H G-buffer on the plane z = 0 (positions on a grid over
  [-5, 5]^2, normal +z, camera at (0, -6, 4)), GGX roughness U[0.1, 0.9],
  albedo U[0.2, 0.8], F0 = 0.02, and quads with side U[0.2, 1.0], centres in
  [-5, 5]^2 x [1, 3], facing down within +-30 degrees, radiance log-U[0.1, 10].
* heightfield: a perspective G-buffer of a seeded fBm heightfield (sum of
  random-phase sine waves, four octaves), roughness U[0.05, 1], convex polygon
  lights with 3..8 vertices and areas log-U[0.01, 1], and random occluder
  triangles (edge U[0.05, 0.5]) in [-6, 6]^2 x [0, 2].

Lights go through the light model of the C ABI (update_polygonal_light and the
std140 packing of write_lights); any library exporting
set_polygonal_light_vertex_count and update_polygonal_light can be passed in.
"""
import ctypes
import os
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _native

GBUFFER_PLANES = 17
F0_DIELECTRIC = 0.02  # shading_pass.frag.glsl:643


@dataclass
class LightSpec:
    """Parameters of one polygonal_light_t before update_polygonal_light."""
    rotation_angles: tuple
    scaling: tuple
    translation: tuple
    radiant_flux: tuple
    plane_vertices: np.ndarray  # (n, 2)


@dataclass
class HostScene:
    width: int
    height: int
    gbuffer: np.ndarray               # float32 [17, H*W]
    primitive: Optional[np.ndarray]   # uint32 [H*W] or None
    lights: np.ndarray                # float32 [N, 12 + 4*maxv], std140 (write_lights)
    max_vertex_count: int
    ltc0: np.ndarray                  # float32 [layers, incl, rough, 4]
    ltc1: np.ndarray                  # float32 [layers, incl, rough, 2]
    ltc_constants: np.ndarray         # float32 [6]
    triangles: np.ndarray             # float32 [T, 9] (v0, v1, v2)
    light_specs: list = field(default_factory=list)

    @property
    def light_count(self):
        return int(self.lights.shape[0])

    @property
    def pixels(self):
        return self.width * self.height


def _normalize(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def build_lights(specs, lib=None):
    """Runs the C light model on each spec and packs the std140 buffer.

    lib: a ctypes library with set_polygonal_light_vertex_count and
    update_polygonal_light (default: the product library).  Slots past a
    light's vertex count hold its vertex 0.
    """
    lib = lib or _native.load()
    maxv = max(3, max(len(s.plane_vertices) for s in specs))
    out = np.zeros((len(specs), 12 + 4 * maxv), np.float32)
    for i, s in enumerate(specs):
        light = _native.PolygonalLight()
        lib.set_polygonal_light_vertex_count(ctypes.byref(light), len(s.plane_vertices))
        for a in range(3):
            light.rotation_angles[a] = s.rotation_angles[a]
            light.translation[a] = s.translation[a]
            light.radiant_flux[a] = s.radiant_flux[a]
        light.scaling_x, light.scaling_y = s.scaling
        for v, (px, py) in enumerate(s.plane_vertices):
            light.vertices_plane_space[4 * v + 0] = float(px)
            light.vertices_plane_space[4 * v + 1] = float(py)
        lib.update_polygonal_light(ctypes.byref(light))
        n = light.vertex_count
        row = out[i]
        row[0:3] = light.surface_radiance[:]
        row[4:8] = light.plane[:]
        row[8:9] = np.array([n], np.uint32).view(np.float32)
        world = np.ctypeslib.as_array(light.vertices_world_space, shape=(4 * n,)).reshape(n, 4)
        for v in range(maxv):
            row[12 + 4 * v:15 + 4 * v] = world[v if v < n else 0, :3]
        lib.destroy_polygonal_light(ctypes.byref(light)) if hasattr(lib, "destroy_polygonal_light") else None
    return out, maxv


def load_quicksave(path):
    """risltc_quick_load: the camera (risltc_camera_t), the lights' std140
    buffer (write_lights layout) and the maximum vertex count of a quicksave
    file (src/main.c:76-125)."""
    lib = _native.load()
    camera = _native.Camera()
    lights = ctypes.POINTER(_native.PolygonalLight)()
    count = ctypes.c_uint32(0)
    _native.check(lib.risltc_quick_load(os.fsencode(path), ctypes.byref(camera), ctypes.byref(lights),
                                        ctypes.byref(count)), "risltc_quick_load")
    try:
        maxv = max(3, int(lib.risltc_max_light_vertex_count(lights, count.value)))
        buf = np.zeros((count.value, 12 + 4 * maxv), np.float32)
        _native.check(lib.risltc_write_lights(buf.ctypes.data_as(_native.c_float_p), lights, count.value, maxv),
                      "risltc_write_lights")
    finally:
        lib.risltc_destroy_lights(lights, count.value)
    return camera, buf, maxv


def resave_quicksave(src, dst):
    """Loads a quicksave file and writes it again with risltc_quick_save."""
    lib = _native.load()
    camera = _native.Camera()
    lights = ctypes.POINTER(_native.PolygonalLight)()
    count = ctypes.c_uint32(0)
    _native.check(lib.risltc_quick_load(os.fsencode(src), ctypes.byref(camera), ctypes.byref(lights),
                                        ctypes.byref(count)), "risltc_quick_load")
    try:
        _native.check(lib.risltc_quick_save(os.fsencode(dst), ctypes.byref(camera), lights, count.value),
                      "risltc_quick_save")
    finally:
        lib.risltc_destroy_lights(lights, count.value)


def light_centers(lights_std140):
    """Mean of each light's world-space vertices (std140 rows)."""
    n = lights_std140[:, 8].view(np.uint32).astype(np.int64)
    maxv = (lights_std140.shape[1] - 12) // 4
    verts = lights_std140[:, 12:12 + 4 * maxv].reshape(-1, maxv, 4)[:, :, :3].astype(np.float64)
    mask = np.arange(maxv)[None, :] < n[:, None]
    return ((verts * mask[:, :, None]).sum(1) / n[:, None]).astype(np.float32)


def cluster_order(lights_std140, cluster_count, seed=0, iterations=32):
    """risltc_cluster_lights on the lights' centres: (order, offsets)."""
    lib = _native.load()
    centers = np.ascontiguousarray(light_centers(lights_std140))
    n = centers.shape[0]
    order = np.zeros(n, np.uint32)
    offsets = np.zeros(cluster_count + 1, np.uint32)
    _native.check(lib.risltc_cluster_lights(centers.ctypes.data_as(_native.c_float_p), n, cluster_count, seed,
                                            iterations, order.ctypes.data_as(_native.c_u32_p),
                                            offsets.ctypes.data_as(_native.c_u32_p)), "risltc_cluster_lights")
    return order, offsets


def cluster_summaries(lights_std140, max_vertex_count, offsets):
    """risltc_cluster_summaries: (bounds [K, 4], power [K]) of lights listed
    cluster by cluster."""
    lib = _native.load()
    lights = np.ascontiguousarray(lights_std140, np.float32)
    offsets = np.ascontiguousarray(offsets, np.uint32)
    k = offsets.size - 1
    bounds = np.zeros((k, 4), np.float32)
    power = np.zeros(k, np.float32)
    _native.check(lib.risltc_cluster_summaries(lights.ctypes.data_as(_native.c_float_p), lights.shape[0],
                                               max_vertex_count, offsets.ctypes.data_as(_native.c_u32_p), k,
                                               bounds.ctypes.data_as(_native.c_float_p),
                                               power.ctypes.data_as(_native.c_float_p)), "risltc_cluster_summaries")
    return bounds, power


def cluster_lights(hs, cluster_count, seed=0, iterations=32):
    """A copy of the scene with its lights (and light specs) listed cluster by
    cluster, and the cluster offsets (cluster c holds lights offsets[c] ..
    offsets[c + 1])."""
    order, offsets = cluster_order(hs.lights, cluster_count, seed, iterations)
    specs = [hs.light_specs[i] for i in order] if hs.light_specs else []
    out = HostScene(hs.width, hs.height, hs.gbuffer, hs.primitive, np.ascontiguousarray(hs.lights[order]),
                    hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants, hs.triangles, specs)
    return out, offsets


def synthetic_ltc(seed=0, size=64):
    """The product's seeded synthetic LTC table (risltc_ltc_table_synthetic)."""
    lib = _native.load()
    t = _native.LtcTable()
    _native.check(lib.risltc_ltc_table_synthetic(ctypes.byref(t), seed, size, size), "synthetic LTC table")
    n = t.roughness_count * t.inclination_count * t.fresnel_count
    ltc0 = np.ctypeslib.as_array(t.texels0, shape=(4 * n,)).copy().reshape(t.fresnel_count, t.inclination_count,
                                                                           t.roughness_count, 4)
    ltc1 = np.ctypeslib.as_array(t.texels1, shape=(2 * n,)).copy().reshape(t.fresnel_count, t.inclination_count,
                                                                           t.roughness_count, 2)
    c = t.constants
    consts = np.array([c.fresnel_index_factor, c.fresnel_index_summand, c.roughness_factor, c.roughness_summand,
                       c.inclination_factor, c.inclination_summand], np.float32)
    lib.risltc_ltc_table_destroy(ctypes.byref(t))
    return ltc0, ltc1, consts


def _gbuffer_planes(pos, nrm, wo, albedo, f0, rough):
    n = pos.shape[0]
    g = np.empty((GBUFFER_PLANES, n), np.float32)
    g[0:3] = pos.T
    g[3:6] = nrm.T
    g[6:9] = wo.T
    g[9] = np.sum(nrm * wo, axis=1, dtype=np.float32)
    g[10:13] = albedo.T
    g[13:16] = f0.T
    g[16] = rough
    return g


def _adapt_normal(nrm, wo):
    """Clip the shading normal into the hemisphere of the view direction
    (shading_pass.frag.glsl:666-670)."""
    off = np.maximum(0.0, 1.0e-3 - np.sum(nrm * wo, axis=1))
    return _normalize(nrm + off[:, None] * wo).astype(np.float32)


def quad_specs(rng, count, center_lo=(-5.0, -5.0, 1.0), center_hi=(5.0, 5.0, 3.0), side=(0.2, 1.0)):
    specs = []
    for _ in range(count):
        s = rng.uniform(*side)
        c = rng.uniform(center_lo, center_hi)
        tilt = np.radians(30.0)
        angles = (np.pi + rng.uniform(-tilt, tilt), rng.uniform(-tilt, tilt), rng.uniform(0.0, 2.0 * np.pi))
        flux = np.exp(rng.uniform(np.log(0.1), np.log(10.0), 3))
        verts = np.array([[-0.5, -0.5], [0.5, -0.5], [0.5, 0.5], [-0.5, 0.5]])
        specs.append(LightSpec(angles, (s, s), tuple(c), tuple(flux), verts))
    return specs


def polygon_specs(rng, count, vertex_counts=(3, 8), area=(0.01, 1.0), center_lo=(-6.0, -6.0, 2.5),
                  center_hi=(6.0, 6.0, 4.0)):
    """Convex polygons inscribed in a circle (jittered regular angles) scaled
    to a log-uniform area."""
    specs = []
    for _ in range(count):
        n = int(rng.integers(vertex_counts[0], vertex_counts[1] + 1))
        base = 2.0 * np.pi * np.arange(n) / n
        ang = base + rng.uniform(-0.35, 0.35, n) * (2.0 * np.pi / n) + rng.uniform(0, 2 * np.pi)
        verts = np.stack([np.cos(ang), np.sin(ang)], axis=1)
        a0 = 0.5 * np.sum(verts[:, 0] * np.roll(verts[:, 1], -1) - np.roll(verts[:, 0], -1) * verts[:, 1])
        target = np.exp(rng.uniform(np.log(area[0]), np.log(area[1])))
        s = np.sqrt(target / a0)
        c = rng.uniform(center_lo, center_hi)
        tilt = np.radians(30.0)
        angles = (np.pi + rng.uniform(-tilt, tilt), rng.uniform(-tilt, tilt), rng.uniform(0.0, 2.0 * np.pi))
        flux = np.exp(rng.uniform(np.log(0.1), np.log(10.0), 3))
        specs.append(LightSpec(angles, (s, s), tuple(c), tuple(flux), verts))
    return specs


def random_triangles(rng, count, lo=(-6.0, -6.0, 0.0), hi=(6.0, 6.0, 2.0), edge=(0.05, 0.5)):
    """Triangles with edge length U[edge] centred uniformly in the box."""
    c = rng.uniform(lo, hi, (count, 3))
    length = rng.uniform(edge[0], edge[1], count)
    a = _normalize(rng.normal(size=(count, 3)))
    b = _normalize(np.cross(a, rng.normal(size=(count, 3))))
    phase = rng.uniform(0, 2 * np.pi, count)
    r = length / np.sqrt(3.0)
    tris = np.empty((count, 3, 3))
    for k in range(3):
        t = phase + 2.0 * np.pi * k / 3.0
        tris[:, k] = c + r[:, None] * (np.cos(t)[:, None] * a + np.sin(t)[:, None] * b)
    return tris.reshape(count, 9).astype(np.float32)


def plane_of_quads(width=256, height=256, light_count=64, seed=0, ltc_size=64, light_lib=None, triangles=0):
    """Configuration 1 (unshadowed unless triangles > 0)."""
    rng = np.random.default_rng(seed)
    xs = (np.arange(width) + 0.5) / width * 10.0 - 5.0
    ys = (np.arange(height) + 0.5) / height * 10.0 - 5.0
    px, py = np.meshgrid(xs, ys)
    pos = np.stack([px.ravel(), py.ravel(), np.zeros(width * height)], axis=1).astype(np.float32)
    nrm = np.tile(np.array([0.0, 0.0, 1.0], np.float32), (pos.shape[0], 1))
    wo = _normalize(np.array([0.0, -6.0, 4.0]) - pos.astype(np.float64)).astype(np.float32)
    rough = rng.uniform(0.1, 0.9, pos.shape[0]).astype(np.float32)
    albedo = rng.uniform(0.2, 0.8, (pos.shape[0], 3)).astype(np.float32)
    f0 = np.full((pos.shape[0], 3), F0_DIELECTRIC, np.float32)
    g = _gbuffer_planes(pos, nrm, wo, albedo, f0, rough)
    specs = quad_specs(rng, light_count)
    lights, maxv = build_lights(specs, light_lib)
    ltc0, ltc1, consts = synthetic_ltc(0, ltc_size)
    tris = random_triangles(rng, triangles, lo=(-5.0, -5.0, 0.05), hi=(5.0, 5.0, 0.9)) if triangles else \
        np.zeros((0, 9), np.float32)
    return HostScene(width, height, g, None, lights, maxv, ltc0, ltc1, consts, tris, specs)


def _heightfield_waves(rng, octaves=4):
    waves = []
    for o in range(octaves):
        amp = 0.25 * 0.5 ** o
        freq = 0.6 * 2.0 ** o
        for _ in range(2):
            d = _normalize(rng.normal(size=2))
            waves.append((amp, freq * d[0], freq * d[1], rng.uniform(0, 2 * np.pi)))
    return np.array(waves, np.float64)


def _height(waves, x, y):
    h = np.zeros_like(x)
    for a, fx, fy, ph in waves.astype(x.dtype):
        h += a * np.sin(fx * x + fy * y + ph)
    return h


def _height_grad(waves, x, y):
    gx = np.zeros_like(x)
    gy = np.zeros_like(x)
    for a, fx, fy, ph in waves:
        c = a * np.cos(fx * x + fy * y + ph)
        gx += c * fx
        gy += c * fy
    return gx, gy


def heightfield_gbuffer_gpu(ctx, width, height, seed=0, camera=(0.0, -9.0, 6.0), fov_y_degrees=60.0,
                            material_seed=None):
    """risltc_gbuffer_heightfield: the heightfield() surface (same waves for
    the same seed) shaded into a G-buffer on the GPU.  Returns (planes
    [17, H*W], primitive [H*W] int32) as torch device tensors.  Materials come
    from a per-pixel hash, not from NumPy's generator."""
    import torch
    rng = np.random.default_rng(seed)
    waves = _heightfield_waves(rng)
    hf = _native.Heightfield()
    for a in range(3):
        hf.camera[a] = camera[a]
    hf.fov_y = float(np.radians(fov_y_degrees))
    hf.wave_count = waves.shape[0]
    for w in range(waves.shape[0]):
        for k in range(4):
            hf.waves[w][k] = float(waves[w, k])
    hf.material_seed = seed if material_seed is None else material_seed
    hf.roughness_min, hf.roughness_max = 0.05, 1.0
    hf.albedo_min, hf.albedo_max = 0.2, 0.8
    hf.fresnel_0 = F0_DIELECTRIC
    planes = torch.empty((GBUFFER_PLANES, width * height), dtype=torch.float32, device="cuda")
    prim = torch.empty(width * height, dtype=torch.int32, device="cuda")
    _native.check(_native.load().risltc_gbuffer_heightfield(ctx.handle, ctypes.byref(hf), width, height,
                                                            ctypes.c_void_p(planes.data_ptr()),
                                                            ctypes.c_void_p(prim.data_ptr())),
                  "risltc_gbuffer_heightfield")
    return planes, prim


def heightfield(width=1920, height=1080, light_count=1024, triangle_count=200_000, seed=0, vertex_counts=(3, 8),
                ltc_size=64, light_lib=None, camera=(0.0, -9.0, 6.0), fov_y_degrees=60.0):
    """Configuration 2: fBm heightfield G-buffer, polygon lights, occluders."""
    rng = np.random.default_rng(seed)
    waves = _heightfield_waves(rng)
    cam = np.array(camera, np.float64)
    fwd = _normalize(-cam)
    right = _normalize(np.cross(fwd, [0.0, 0.0, 1.0]))
    up = np.cross(right, fwd)
    th = np.tan(np.radians(fov_y_degrees) / 2.0)
    tw = th * width / height
    u = ((np.arange(width) + 0.5) / width * 2.0 - 1.0) * tw
    v = (1.0 - (np.arange(height) + 0.5) / height * 2.0) * th
    uu, vv = np.meshgrid(u, v)
    d = _normalize(fwd[None, :] + uu.reshape(-1, 1) * right[None, :] + vv.reshape(-1, 1) * up[None, :])
    hmax = np.sum(np.abs(waves[:, 0]))
    valid = d[:, 2] < -1e-3
    dz = np.where(valid, d[:, 2], -1.0)
    t_lo = (cam[2] - hmax) / -dz
    t_hi = (cam[2] + hmax) / -dz

    d32 = d.astype(np.float32)
    cam32 = cam.astype(np.float32)

    def g(t):
        t = t.astype(np.float32)
        x = cam32[0] + t * d32[:, 0]
        y = cam32[1] + t * d32[:, 1]
        z = cam32[2] + t * d32[:, 2]
        return z - _height(waves, x, y)

    # Coarse march for the first sign change, then bisection.
    steps = 10
    a = t_lo.copy()
    b = t_hi.copy()
    found = np.zeros(a.shape, bool)
    prev_t = t_lo.copy()
    for k in range(1, steps + 1):
        t = t_lo + (t_hi - t_lo) * k / steps
        below = (g(t) <= 0.0) & ~found
        a = np.where(below, prev_t, a)
        b = np.where(below, t, b)
        found |= below
        prev_t = t
    for _ in range(12):
        m = 0.5 * (a + b)
        below = g(m) <= 0.0
        b = np.where(below, m, b)
        a = np.where(below, a, m)
    t = 0.5 * (a + b)
    pos = (cam[None, :] + t[:, None] * d)
    gx, gy = _height_grad(waves, pos[:, 0], pos[:, 1])
    nrm = _normalize(np.stack([-gx, -gy, np.ones_like(gx)], axis=1))
    wo = _normalize(cam[None, :] - pos)
    nrm = _adapt_normal(nrm, wo)
    n = width * height
    rough = rng.uniform(0.05, 1.0, n).astype(np.float32)
    albedo = rng.uniform(0.2, 0.8, (n, 3)).astype(np.float32)
    f0 = np.full((n, 3), F0_DIELECTRIC, np.float32)
    gb = _gbuffer_planes(pos.astype(np.float32), nrm.astype(np.float32), wo.astype(np.float32), albedo, f0, rough)
    primitive = np.where(valid & found, 0, 0xFFFFFFFF).astype(np.uint32)
    specs = polygon_specs(rng, light_count, vertex_counts)
    lights, maxv = build_lights(specs, light_lib)
    ltc0, ltc1, consts = synthetic_ltc(0, ltc_size)
    tris = random_triangles(rng, triangle_count) if triangle_count else np.zeros((0, 9), np.float32)
    return HostScene(width, height, gb, primitive, lights, maxv, ltc0, ltc1, consts, tris, specs)
