"""Python access to the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

TECHNIQUE = {"ltc_cp": 4, "projected_solid_angle": 2, "projected_solid_angle_biased": 3, "area_turk": 1}
MIS = {"balance": 0, "power": 1, "weighted": 2, "optimal_clamped": 3, "optimal": 4}
LIGHT_SAMPLING = {"uniform": 0, "ris": 1}


class Scene(ctypes.Structure):
    _fields_ = [("lights", ctypes.c_void_p), ("light_count", ctypes.c_int32),
                ("max_light_vertex_count", ctypes.c_int32), ("ltc0", ctypes.c_void_p), ("ltc1", ctypes.c_void_p),
                ("ltc_width", ctypes.c_int32), ("ltc_height", ctypes.c_int32), ("ltc_layers", ctypes.c_int32),
                ("ltc_constants", ctypes.c_float * 6), ("triangles", ctypes.c_void_p),
                ("triangle_count", ctypes.c_int32), ("bvh_nodes", ctypes.c_void_p), ("bvh_node_count", ctypes.c_int32),
                ("cluster_offsets", ctypes.c_void_p), ("light_cluster", ctypes.c_void_p),
                ("cluster_bounds", ctypes.c_void_p), ("cluster_power", ctypes.c_void_p),
                ("cluster_count", ctypes.c_int32)]


class Settings(ctypes.Structure):
    _fields_ = [("polygon_sampling_technique", ctypes.c_int32), ("light_sampling", ctypes.c_int32),
                ("mis_heuristic", ctypes.c_int32), ("candidate_count", ctypes.c_int32),
                ("sample_count", ctypes.c_int32), ("light_samples", ctypes.c_int32),
                ("mis_visibility_estimate", ctypes.c_float), ("fast_atan", ctypes.c_int32),
                ("reference_slots", ctypes.c_int32), ("proposal", ctypes.c_int32),
                ("proposal_uniform_fraction", ctypes.c_float), ("random_number_proposal", ctypes.c_uint32)]


class GBuffer(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("planes", ctypes.c_void_p),
                ("primitive", ctypes.c_void_p)]


class Reservoir(ctypes.Structure):
    _fields_ = [("light_index", ctypes.c_int32), ("pad", ctypes.c_int32), ("w_sum", ctypes.c_double),
                ("sample_value", ctypes.c_double)]


RESERVOIR_DTYPE = np.dtype([("light_index", np.int32), ("pad", np.int32), ("w_sum", np.float64),
                            ("sample_value", np.float64)])

_lib = None


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build_oracle.build())
        args = [ctypes.POINTER(Scene), ctypes.POINTER(Settings), ctypes.POINTER(GBuffer), ctypes.c_uint32,
                ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.oracle_render_f32.argtypes = args
        lib.oracle_render_f64.argtypes = args
        lib.oracle_render_frame_f32.argtypes = args[:4] + [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                          ctypes.c_void_p, ctypes.c_void_p,
                                                          ctypes.POINTER(ctypes.c_double)]
        lib.oracle_render_pixels_omp_f32.argtypes = args[:4] + [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                                ctypes.c_void_p, ctypes.c_void_p,
                                                                ctypes.POINTER(ctypes.c_double)]
        lib.oracle_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


class OracleScene:
    """Keeps the numpy arrays alive while the C structs point into them."""

    def __init__(self, lights, max_vertex_count, ltc0, ltc1, ltc_constants, triangles_v0e1e2=None, bvh_nodes=None):
        self.lights = np.ascontiguousarray(lights, np.float32)
        self.ltc0 = np.ascontiguousarray(ltc0, np.float32)
        self.ltc1 = np.ascontiguousarray(ltc1, np.float32)
        self.tris = None if triangles_v0e1e2 is None else np.ascontiguousarray(triangles_v0e1e2, np.float32)
        self.nodes = None if bvh_nodes is None else np.ascontiguousarray(bvh_nodes, np.float32)
        s = Scene()
        s.lights = self.lights.ctypes.data
        s.light_count = self.lights.shape[0]
        s.max_light_vertex_count = max_vertex_count
        s.ltc0 = self.ltc0.ctypes.data
        s.ltc1 = self.ltc1.ctypes.data
        s.ltc_layers, s.ltc_height, s.ltc_width = self.ltc0.shape[:3]
        for i in range(6):
            s.ltc_constants[i] = float(ltc_constants[i])
        if self.tris is not None and len(self.tris):
            s.triangles = self.tris.ctypes.data
            s.triangle_count = self.tris.shape[0]
        if self.nodes is not None:
            s.bvh_nodes = self.nodes.ctypes.data
            s.bvh_node_count = self.nodes.shape[0]
        self.struct = s

    def set_clusters(self, offsets, bounds, power):
        """Cluster structure for the proposal: offsets (count + 1), bounds
        (count x 4: centre, radius) and power (count), as the product
        computes them (risltc_cluster_summaries)."""
        self.offsets = np.ascontiguousarray(offsets, np.uint32)
        self.bounds = np.ascontiguousarray(bounds, np.float32)
        self.power = np.ascontiguousarray(power, np.float32)
        count = self.offsets.size - 1
        self.light_cluster = np.repeat(np.arange(count, dtype=np.uint32), np.diff(self.offsets.astype(np.int64)))
        s = self.struct
        s.cluster_offsets = self.offsets.ctypes.data
        s.light_cluster = self.light_cluster.ctypes.data
        s.cluster_bounds = self.bounds.ctypes.data
        s.cluster_power = self.power.ctypes.data
        s.cluster_count = count


def triangles_v0e1e2(tris9):
    """(v0, v1, v2) rows to the 12-float {v0, 0, v1 - v0, 0, v2 - v0, 0} layout."""
    t = np.asarray(tris9, np.float32).reshape(-1, 3, 3)
    out = np.zeros((t.shape[0], 12), np.float32)
    out[:, 0:3] = t[:, 0]
    out[:, 4:7] = t[:, 1] - t[:, 0]
    out[:, 8:11] = t[:, 2] - t[:, 0]
    return out


def make_settings(technique="ltc_cp", light_sampling="ris", mis="optimal_clamped", candidates=32, sample_count=1,
                  light_samples=1, mis_visibility_estimate=0.5, fast_atan=False, reference_slots=False,
                  proposal=False, proposal_uniform_fraction=0.1, random_number_proposal=0):
    s = Settings()
    s.polygon_sampling_technique = TECHNIQUE[technique]
    s.light_sampling = LIGHT_SAMPLING[light_sampling]
    s.mis_heuristic = MIS[mis]
    s.candidate_count = candidates
    s.sample_count = sample_count
    s.light_samples = light_samples
    s.mis_visibility_estimate = mis_visibility_estimate
    s.fast_atan = int(fast_atan)
    s.reference_slots = int(reference_slots)
    s.proposal = int(proposal)
    s.proposal_uniform_fraction = proposal_uniform_fraction
    s.random_number_proposal = random_number_proposal
    return s


def render(scene, settings, gbuffer, width, height, random_number_x, primitive=None, precision="f32",
           rows=None, threads=0, reservoirs=True):
    """Renders one frame; returns (rgb [H*W, 3], reservoirs or None, seconds)."""
    lib = load()
    g = GBuffer()
    g.width, g.height = width, height
    gbuffer = np.ascontiguousarray(gbuffer, np.float32)
    g.planes = gbuffer.ctypes.data
    prim = None if primitive is None else np.ascontiguousarray(primitive, np.uint32)
    g.primitive = None if prim is None else prim.ctypes.data
    r0, r1 = (0, height) if rows is None else rows
    dtype = np.float32 if precision == "f32" else np.float64
    rgb = np.zeros((width * height, 3), dtype)
    res = np.zeros(width * height, RESERVOIR_DTYPE) if reservoirs else None
    res_ptr = None if res is None else res.ctypes.data
    seconds = ctypes.c_double(0.0)
    if precision == "f32":
        status = lib.oracle_render_frame_f32(ctypes.byref(scene.struct), ctypes.byref(settings), ctypes.byref(g),
                                             random_number_x, threads, r0, r1, rgb.ctypes.data, res_ptr,
                                             ctypes.byref(seconds))
    else:
        status = lib.oracle_render_f64(ctypes.byref(scene.struct), ctypes.byref(settings), ctypes.byref(g),
                                       random_number_x, r0, r1, rgb.ctypes.data, res_ptr)
    if status != 0:
        raise RuntimeError("oracle render failed (status %d)" % status)
    return rgb, res, seconds.value


def render_pixels(scene, settings, gbuffer, width, height, random_number_x, pixels, primitive=None, threads=0,
                  reservoirs=True):
    """Renders the listed pixels (indices y * width + x) of a full frame, each
    with its own position's noise seed, in FP32.  Returns (rgb [K, 3],
    reservoirs [K] or None, seconds): row k belongs to pixels[k]."""
    lib = load()
    g = GBuffer()
    g.width, g.height = width, height
    gbuffer = np.ascontiguousarray(gbuffer, np.float32)
    assert gbuffer.shape == (17, width * height)
    g.planes = gbuffer.ctypes.data
    prim = None if primitive is None else np.ascontiguousarray(primitive, np.uint32)
    g.primitive = None if prim is None else prim.ctypes.data
    px = np.ascontiguousarray(pixels, np.uint32)
    assert px.size == 0 or int(px.max()) < width * height
    rgb = np.zeros((px.size, 3), np.float32)
    res = np.zeros(px.size, RESERVOIR_DTYPE) if reservoirs else None
    seconds = ctypes.c_double(0.0)
    status = lib.oracle_render_pixels_omp_f32(ctypes.byref(scene.struct), ctypes.byref(settings), ctypes.byref(g),
                                              random_number_x, px.ctypes.data, int(px.size), threads, rgb.ctypes.data,
                                              None if res is None else res.ctypes.data, ctypes.byref(seconds))
    if status != 0:
        raise RuntimeError("oracle render failed (status %d)" % status)
    return rgb, res, seconds.value


class OpCounts(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("add", "mul", "fma", "div", "sqrt", "atan", "sincos", "acos", "cmp",
                                               "boxes", "triangles")]


# FP32 operations inside one call of each transcendental of include/risltc_math.h
# (its polynomial evaluation plus reduction), counted from the source.
TRANSCENDENTAL_FLOPS = {"atan": 24, "sincos": 30, "acos": 29}

_oplib = None


def opcount(scene, settings, gbuffer, width, height, random_number_x, rows, primitive=None):
    """Renders rows with the op-counting oracle; returns a dict of tallies
    and 'flops' = add + mul + 2 fma + div + sqrt + transcendental flops."""
    global _oplib
    if _oplib is None:
        build_oracle.build()
        _oplib = ctypes.CDLL(build_oracle.OPCOUNT_LIB)
        _oplib.oracle_opcount_render.argtypes = [ctypes.POINTER(Scene), ctypes.POINTER(Settings),
                                                 ctypes.POINTER(GBuffer), ctypes.c_uint32, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(OpCounts)]
    g = GBuffer()
    g.width, g.height = width, height
    gbuffer = np.ascontiguousarray(gbuffer, np.float32)
    g.planes = gbuffer.ctypes.data
    prim = None if primitive is None else np.ascontiguousarray(primitive, np.uint32)
    g.primitive = None if prim is None else prim.ctypes.data
    rgb = np.zeros((width * height, 3), np.float32)
    c = OpCounts()
    if _oplib.oracle_opcount_render(ctypes.byref(scene.struct), ctypes.byref(settings), ctypes.byref(g),
                                    random_number_x, rows[0], rows[1], rgb.ctypes.data, ctypes.byref(c)) != 0:
        raise RuntimeError("op-count render failed")
    d = {k: int(getattr(c, k)) for k, _ in OpCounts._fields_}
    d["flops"] = (d["add"] + d["mul"] + 2 * d["fma"] + d["div"] + d["sqrt"]
                  + sum(d[k] * v for k, v in TRANSCENDENTAL_FLOPS.items()))
    d["rgb"] = rgb
    return d


def max_threads():
    return load().oracle_max_threads()
