"""Python front end of the C ABI (include/risltc.h).

Mirrors the reference's per-frame flow (render_frame, src/main.c:2955-3041):
build lights with the polygonal-light model, load an LTC table, set the noise
constants, then shade the frame's G-buffer.  Device buffers are torch CUDA
tensors (PyTorch supplies memory and streams only); host buffers are numpy.
Every call goes through librisltc_gb300.so and raises RisltcError on failure.
There is no CPU fallback.
"""
import ctypes

import numpy as np

from . import _native
from ._native import RisltcError, check  # noqa: F401

TECHNIQUES = {"baseline": 0, "area_turk": 1, "projected_solid_angle": 2, "projected_solid_angle_biased": 3,
              "ltc_cp": 4}
MIS_HEURISTICS = {"balance": 0, "power": 1, "weighted": 2, "optimal_clamped": 3, "optimal": 4}
LIGHT_SAMPLING = {"uniform": 0, "ris": 1}
NUMERICS = {"exact": 0, "fast": 1}
PROPOSALS = {"uniform": 0, "clusters": 1, "learned": 2}
# risltc_tile_t: candidate kernel tile shapes (pixels per warp x candidates
# per pixel per chunk, or one thread per pixel), in enum order.
TILES = {"32x8": 0, "16x8": 1, "8x8": 2, "32x4": 3, "16x4": 4, "per_pixel": 5}
TILE_NAMES = {v: k for k, v in TILES.items()}


def settings(technique="ltc_cp", light_sampling="ris", mis="optimal_clamped", candidates=32, sample_count=1,
             light_samples=1, mis_visibility_estimate=0.5, fast_atan=False, shadows=True, numerics="exact",
             proposal="uniform", proposal_uniform_fraction=0.1, tile="32x8"):
    """risltc_settings_t; defaults are specify_default_render_settings
    (src/main.c:220-236) with the reference's hard-coded M = 32."""
    s = _native.Settings()
    _native.load().risltc_default_settings(ctypes.byref(s))
    s.polygon_sampling_technique = TECHNIQUES[technique]
    s.light_sampling = LIGHT_SAMPLING[light_sampling]
    s.mis_heuristic = MIS_HEURISTICS[mis]
    s.candidate_count = candidates
    s.sample_count = sample_count
    s.sample_count_light = light_samples
    s.mis_visibility_estimate = mis_visibility_estimate
    s.fast_atan = int(fast_atan)
    s.shadows = int(shadows)
    s.numerics = NUMERICS[numerics]
    s.proposal = PROPOSALS[proposal]
    s.proposal_uniform_fraction = proposal_uniform_fraction
    s.tile = TILES[tile]
    return s


def copy_settings(s, **changes):
    """A copy of risltc_settings_t s with fields replaced (tile by name)."""
    out = _native.Settings()
    ctypes.pointer(out)[0] = s
    for k, v in changes.items():
        setattr(out, k, TILES[v] if k == "tile" else v)
    return out


def noise_constants(frame, animate=True):
    """random_numbers[4] of set_noise_constants for the given frame index."""
    lib = _native.load()
    rn = (ctypes.c_uint32 * 4)()
    nt = _native.NoiseTable(frame)
    lib.set_noise_constants(None, None, rn, ctypes.byref(nt), int(animate))
    return list(rn)


class Context:
    """risltc_ctx_t: one device, one stream (default: torch's current stream)."""

    def __init__(self, device=0, stream=None):
        self._lib = _native.load()
        if stream is None:
            try:
                import torch
                stream = torch.cuda.current_stream(device).cuda_stream
            except Exception:  # noqa: BLE001 - no torch CUDA: legacy default stream
                stream = 0
        self._h = ctypes.c_void_p()
        check(self._lib.risltc_ctx_create(ctypes.byref(self._h), device, ctypes.c_void_p(stream)), "risltc_ctx_create")
        self.device = device
        # (destroy function, handle) of the scenes and models made on this
        # context: closing it destroys them first, whatever order the
        # interpreter runs finalizers in at exit (a finalizer of a garbage
        # cycle may run before those of the objects that refer to it).
        self._owned = []

    def _adopt(self, destroy, handle):
        self._owned.append((destroy, handle))

    @property
    def handle(self):
        return self._h

    def check(self):
        check(self._lib.risltc_ctx_check(self._h), "risltc_ctx_check")

    def inject_fault(self, tensor_wait=False, train_tensor_wait=False):
        """risltc_ctx_inject_fault: host-made faults for tests of the failure
        paths (see include/risltc.h): the next logits launch (tensor_wait) or
        tensor-core training launch (train_tensor_wait) issues no products."""
        faults = (1 if tensor_wait else 0) | (2 if train_tensor_wait else 0)
        check(self._lib.risltc_ctx_inject_fault(self._h, faults), "risltc_ctx_inject_fault")

    def profile(self, enable=True):
        """Per-kernel CUDA-event times (ms) of the shading calls since the last
        call, then switches timing on or off.  Returns a dict: candidates
        (or the fused kernel), shade, ray_sort (bucket scan and scatter),
        shadow_trace and resolve (0 where the phase is not a kernel of its
        own), and calls."""
        ms = (ctypes.c_float * 5)()
        calls = ctypes.c_uint32(0)
        check(self._lib.risltc_ctx_profile(self._h, int(enable), ms, ctypes.byref(calls)), "risltc_ctx_profile")
        return dict(candidates=float(ms[0]), shade=float(ms[1]), ray_sort=float(ms[2]), shadow_trace=float(ms[3]),
                    resolve=float(ms[4]), calls=int(calls.value))

    def launch_count(self):
        """risltc_ctx_launch_count: this library's kernels launched so far."""
        n = ctypes.c_uint64(0)
        check(self._lib.risltc_ctx_launch_count(self._h, ctypes.byref(n)), "risltc_ctx_launch_count")
        return int(n.value)

    def ray_count(self):
        """risltc_ctx_ray_count: shadow rays the last risltc_shade call traced
        through its ray queue (0 if it traced none that way)."""
        n = ctypes.c_uint32(0)
        check(self._lib.risltc_ctx_ray_count(self._h, ctypes.byref(n)), "risltc_ctx_ray_count")
        return int(n.value)

    def close(self):
        if self._h:
            for destroy, handle in reversed(self._owned):
                if handle:
                    destroy(handle)
                    handle.value = None
            self._owned.clear()
            self._lib.risltc_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


class Scene:
    """risltc_scene_t: lights, LTC table and occluder BVH resident on the device."""

    def __init__(self, ctx, lights_std140, max_vertex_count, ltc0, ltc1, ltc_constants, triangles=None):
        self._lib = _native.load()
        self.ctx = ctx
        lights = np.ascontiguousarray(lights_std140, np.float32)
        ltc0 = np.ascontiguousarray(ltc0, np.float32)
        ltc1 = np.ascontiguousarray(ltc1, np.float32)
        table = _native.LtcTable()
        table.fresnel_count, table.inclination_count, table.roughness_count = ltc0.shape[:3]
        table.texels0 = ltc0.ctypes.data_as(_native.c_float_p)
        table.texels1 = ltc1.ctypes.data_as(_native.c_float_p)
        c = table.constants
        (c.fresnel_index_factor, c.fresnel_index_summand, c.roughness_factor, c.roughness_summand,
         c.inclination_factor, c.inclination_summand) = [float(x) for x in ltc_constants[:6]]
        tris = None if triangles is None or len(triangles) == 0 else np.ascontiguousarray(triangles, np.float32)
        self._h = ctypes.c_void_p()
        check(self._lib.risltc_scene_create(
            ctx.handle, lights.ctypes.data_as(_native.c_float_p), lights.shape[0], max_vertex_count,
            ctypes.byref(table), None if tris is None else tris.ctypes.data_as(_native.c_float_p),
            0 if tris is None else tris.shape[0], ctypes.byref(self._h)), "risltc_scene_create")
        ctx._adopt(self._lib.risltc_scene_destroy, self._h)
        self.light_count = lights.shape[0]

    @classmethod
    def from_host_scene(cls, ctx, hs, shadows=True):
        return cls(ctx, hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants,
                   hs.triangles if shadows else None)

    def set_model(self, model):
        """risltc_scene_set_model (None detaches)."""
        check(self._lib.risltc_scene_set_model(self._h, None if model is None else model.handle),
              "risltc_scene_set_model")

    def set_clusters(self, offsets):
        """risltc_scene_set_clusters: the lights must be listed cluster by
        cluster (scenes.cluster_lights)."""
        off = np.ascontiguousarray(offsets, np.uint32)
        check(self._lib.risltc_scene_set_clusters(self._h, off.ctypes.data_as(_native.c_u32_p), off.size - 1),
              "risltc_scene_set_clusters")

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            self._lib.risltc_scene_destroy(self._h)
            self._h.value = None  # also in the context's list

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


class Model:
    """risltc_model_t: the learned cluster proposal's MLP (see include/risltc.h)."""

    def __init__(self, ctx, cluster_count, seed=0):
        self._lib = _native.load()
        self.ctx = ctx
        self.cluster_count = cluster_count
        self._h = ctypes.c_void_p()
        check(self._lib.risltc_model_create(ctx.handle, cluster_count, seed, ctypes.byref(self._h)),
              "risltc_model_create")
        ctx._adopt(self._lib.risltc_model_destroy, self._h)

    @property
    def handle(self):
        return self._h

    @property
    def parameter_count(self):
        return int(self._lib.risltc_model_parameter_count(self.cluster_count))

    def get_params(self):
        out = np.zeros(self.parameter_count, np.float32)
        check(self._lib.risltc_model_get_params(self._h, out.ctypes.data_as(_native.c_float_p)),
              "risltc_model_get_params")
        return out

    def set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == self.parameter_count
        check(self._lib.risltc_model_set_params(self._h, p.ctypes.data_as(_native.c_float_p)),
              "risltc_model_set_params")

    def set_training(self, enable=True, learning_rate=1e-3, pixel_stride=64):
        check(self._lib.risltc_model_set_training(self._h, int(enable), learning_rate, pixel_stride),
              "risltc_model_set_training")

    def set_target_mix(self, shadowed_weight):
        check(self._lib.risltc_model_set_target_mix(self._h, float(shadowed_weight)), "risltc_model_set_target_mix")

    TRAIN_CUDA_CORES = 1
    TRAIN_ACCUMULATE_ONLY = 2

    def set_training_flags(self, cuda_cores=False, accumulate_only=False):
        """risltc_model_set_training_flags: cuda_cores trains with the FP32
        CUDA-core kernel instead of the tensor cores; accumulate_only adds each
        step's gradient without an Adam step (apply_update takes it)."""
        flags = (self.TRAIN_CUDA_CORES if cuda_cores else 0) | (self.TRAIN_ACCUMULATE_ONLY if accumulate_only else 0)
        check(self._lib.risltc_model_set_training_flags(self._h, flags), "risltc_model_set_training_flags")

    def get_gradient(self, clear=False):
        out = np.zeros(self.parameter_count, np.float32)
        check(self._lib.risltc_model_get_gradient(self._h, out.ctypes.data_as(_native.c_float_p), int(clear)),
              "risltc_model_get_gradient")
        return out

    def train(self, scene, gbuffer, width, height, candidates, stride, phase=0, shaded=None, reservoirs=None,
              primitive=None):
        """risltc_model_train: one training step on caller-supplied candidates.
        candidates: device tensor of width * height * M (light, weight) pairs
        (int32 [P, M, 2] with the weights' bits in the second column, or
        float32 viewed alike); shaded: float32 [P] and reservoirs: int32
        [P, 4] (device) for the shadowed part, or None."""
        m = candidates.shape[1]
        g = _native.GBuffer(width, height, gbuffer.data_ptr(), None if primitive is None else primitive.data_ptr())
        ptr = (lambda t: None if t is None else ctypes.c_void_p(t.data_ptr()))
        check(self._lib.risltc_model_train(self.ctx.handle, scene.handle, ctypes.byref(g), ptr(candidates), m, stride,
                                           phase, ptr(shaded), ptr(reservoirs)), "risltc_model_train")

    def apply_update(self):
        check(self._lib.risltc_model_apply_update(self._h), "risltc_model_apply_update")

    def set_input_transform(self, center, half_extent):
        c = np.ascontiguousarray(center, np.float32)
        check(self._lib.risltc_model_set_input_transform(self._h, c.ctypes.data_as(_native.c_float_p),
                                                         float(half_extent)), "risltc_model_set_input_transform")

    def logits(self, gbuffer, width, height, primitive=None):
        """Device tensor [width*height, clusters] of the model's logits."""
        import torch
        out = torch.empty((width * height, self.cluster_count), dtype=torch.float32, device=gbuffer.device)
        g = _native.GBuffer(width, height, gbuffer.data_ptr(), None if primitive is None else primitive.data_ptr())
        check(self._lib.risltc_model_logits(self.ctx.handle, self._h, ctypes.byref(g), ctypes.c_void_p(out.data_ptr())),
              "risltc_model_logits")
        return out

    def close(self):
        if self._h:
            self._lib.risltc_model_destroy(self._h)
            self._h.value = None  # also in the context's list

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def shade(ctx, scene, gbuffer, width, height, s, noise_seed=0, animate=True, frames=1, out_rgb=None, accum=None,
          reservoirs=None, primitive=None):
    """risltc_shade on device tensors.  gbuffer: float32 [17, H*W] on the GPU;
    out_rgb: float32 [H*W, 3]; accum: float64 [H*W, 3]; reservoirs: int32
    [H*W, 4] viewed as risltc_reservoir_t.  Returns the next noise seed."""
    lib = _native.load()
    g = _native.GBuffer(width, height, gbuffer.data_ptr(), None if primitive is None else primitive.data_ptr())
    nt = _native.NoiseTable(noise_seed)
    ptr = (lambda t: None if t is None else ctypes.c_void_p(t.data_ptr()))
    check(lib.risltc_shade(ctx.handle, scene.handle, ctypes.byref(g), ctypes.byref(s), ctypes.byref(nt), int(animate),
                           frames, ptr(out_rgb), ptr(accum), ptr(reservoirs)), "risltc_shade")
    return nt.random_seed


def _batch_array(items):
    arr = (_native.BatchItem * len(items))()
    tables = [_native.NoiseTable(it.get("noise_seed", 0)) for it in items]
    ptr = (lambda t: None if t is None else t.data_ptr())
    for a, it, nt in zip(arr, items, tables):
        a.scene = it["scene"].handle.value
        prim = it.get("primitive")
        a.gbuffer = _native.GBuffer(it["width"], it["height"], it["gbuffer"].data_ptr(), ptr(prim))
        a.settings = it["settings"]
        a.noise = ctypes.pointer(nt)
        a.animate = int(it.get("animate", True))
        a.frame_count = it.get("frames", 1)
        a.out_rgb, a.accum, a.reservoirs = ptr(it.get("out_rgb")), ptr(it.get("accum")), ptr(it.get("reservoirs"))
    return arr, tables


def shade_batch(ctx, items):
    """risltc_shade_batch.  items: dicts with the keyword arguments of shade()
    (scene, gbuffer, width, height, settings, noise_seed, animate, frames,
    out_rgb, accum, reservoirs, primitive).  Returns each item's next noise
    seed."""
    arr, tables = _batch_array(items)
    check(_native.load().risltc_shade_batch(ctx.handle, arr, len(items)), "risltc_shade_batch")
    return [nt.random_seed for nt in tables]


def autotune(ctx, scene, gbuffer, width, height, s, noise_seed=0, frames=1, repeats=3, primitive=None):
    """risltc_autotune: times the candidate kernel of this shade() call with
    every tile shape.  Returns (a copy of s with the fastest tile, {tile name:
    mean ms per call})."""
    lib = _native.load()
    g = _native.GBuffer(width, height, gbuffer.data_ptr(), None if primitive is None else primitive.data_ptr())
    tuned = copy_settings(s)
    nt = _native.NoiseTable(noise_seed)
    ms = (ctypes.c_float * len(TILES))()
    check(lib.risltc_autotune(ctx.handle, scene.handle, ctypes.byref(g), ctypes.byref(tuned), ctypes.byref(nt),
                              frames, repeats, ms), "risltc_autotune")
    return tuned, {TILE_NAMES[t]: ms[t] for t in range(len(TILES))}


def autotune_batch(ctx, items, repeats=3):
    """risltc_autotune_batch: times the whole shade_batch(ctx, items) call with
    every tile shape and stores a copy of each item's settings with the
    fastest tile in items[i]["settings"].  Returns (tile name, {tile name:
    mean ms per batch})."""
    arr, _ = _batch_array(items)
    ms = (ctypes.c_float * len(TILES))()
    check(_native.load().risltc_autotune_batch(ctx.handle, arr, len(items), repeats, ms), "risltc_autotune_batch")
    for it, a in zip(items, arr):
        it["settings"] = copy_settings(a.settings)
    return TILE_NAMES[arr[0].settings.tile], {TILE_NAMES[t]: ms[t] for t in range(len(TILES))}


def shade_host(ctx, scene, gbuffer, width, height, s, noise_seed=0, animate=True, frames=1, primitive=None,
               out=None):
    """risltc_shade_host: numpy in, numpy out (copies and synchronisation inside)."""
    lib = _native.load()
    g = np.ascontiguousarray(gbuffer, np.float32)
    if out is None:
        out = np.empty((width * height, 3), np.float32)
    prim = None if primitive is None else np.ascontiguousarray(primitive, np.uint32)
    nt = _native.NoiseTable(noise_seed)
    check(lib.risltc_shade_host(ctx.handle, scene.handle, width, height, g.ctypes.data_as(_native.c_float_p),
                                None if prim is None else prim.ctypes.data_as(_native.c_u32_p), ctypes.byref(s),
                                ctypes.byref(nt), int(animate), frames, out.ctypes.data_as(_native.c_float_p)),
          "risltc_shade_host")
    return out


def trace_shadow(ctx, scene, rays, hits):
    """risltc_trace_shadow: rays float32 [R, 8] and hits uint32 [R] on the GPU."""
    check(_native.load().risltc_trace_shadow(ctx.handle, scene.handle, ctypes.c_void_p(rays.data_ptr()),
                                             rays.shape[0], ctypes.c_void_p(hits.data_ptr())), "risltc_trace_shadow")


def build_bvh(triangles, max_leaf_size=4):
    """Host SAH BVH (risltc_bvh_build): returns (nodes [N, 8] float32 with int
    words, triangles [T, 12] float32, triangle_ids [T], depth)."""
    lib = _native.load()
    tris = np.ascontiguousarray(triangles, np.float32)
    b = _native.Bvh()
    check(lib.risltc_bvh_build(ctypes.byref(b), tris.ctypes.data_as(_native.c_float_p), tris.shape[0],
                               max_leaf_size), "risltc_bvh_build")
    try:
        if b.node_count == 0:
            return np.zeros((0, 8), np.float32), np.zeros((0, 12), np.float32), np.zeros(0, np.uint32), 0
        nodes = np.ctypeslib.as_array(b.nodes, shape=(b.node_count * 8,)).copy().reshape(-1, 8)
        t = np.ctypeslib.as_array(b.triangles, shape=(b.triangle_count * 12,)).copy().reshape(-1, 12)
        ids = np.ctypeslib.as_array(b.triangle_ids, shape=(b.triangle_count,)).copy()
        return nodes, t, ids, b.depth
    finally:
        lib.risltc_bvh_destroy(ctypes.byref(b))
