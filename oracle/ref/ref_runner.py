"""Runs the compiled reference shading pass (oracle/_ref/ref_shading_pass_*.so).

TEST INFRASTRUCTURE, used only in the container that holds the reference
sources, by tests/golden/make_golden.py.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_ref  # noqa: E402


class RefInputs(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("gbuffer", ctypes.c_void_p),
                ("primitive", ctypes.c_void_p), ("lights", ctypes.c_void_p), ("light_count", ctypes.c_int),
                ("ltc0", ctypes.c_void_p), ("ltc1", ctypes.c_void_p), ("ltc_width", ctypes.c_int),
                ("ltc_height", ctypes.c_int), ("ltc_layers", ctypes.c_int), ("ltc_constants", ctypes.c_float * 6),
                ("noise_random_numbers", ctypes.c_uint32 * 4), ("mis_visibility_estimate", ctypes.c_float),
                ("triangles", ctypes.c_void_p), ("triangle_count", ctypes.c_int)]


def render(cfg, width, height, gbuffer, lights, ltc0, ltc1, ltc_constants, random_numbers, triangles9=None,
           primitive=None, mis_visibility_estimate=0.5):
    """Shades one frame with the reference's own shader code.

    cfg: shader specialisation (see build_ref._defines); cfg["maxv"] must equal
    the light buffer's vertex slots.  Returns (rgb [P, 3], reads [P, 2]).
    """
    lib = ctypes.CDLL(build_ref.build_ref(cfg))
    lib.ref_render.argtypes = [ctypes.POINTER(RefInputs), ctypes.c_void_p, ctypes.c_void_p]
    keep = []

    def ptr(a, dtype):
        a = np.ascontiguousarray(a, dtype)
        keep.append(a)
        return a.ctypes.data

    inp = RefInputs()
    inp.width, inp.height = width, height
    inp.gbuffer = ptr(gbuffer, np.float32)
    inp.primitive = None if primitive is None else ptr(primitive, np.uint32)
    inp.lights = ptr(lights, np.float32)
    inp.light_count = lights.shape[0]
    inp.ltc0 = ptr(ltc0, np.float32)
    inp.ltc1 = ptr(ltc1, np.float32)
    inp.ltc_layers, inp.ltc_height, inp.ltc_width = ltc0.shape[:3]
    for i in range(6):
        inp.ltc_constants[i] = float(ltc_constants[i])
    for i in range(4):
        inp.noise_random_numbers[i] = int(random_numbers[i])
    inp.mis_visibility_estimate = mis_visibility_estimate
    if triangles9 is not None and len(triangles9):
        t = np.asarray(triangles9, np.float32).reshape(-1, 3, 3)
        v0e1e2 = np.concatenate([t[:, 0], t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]], axis=1)
        inp.triangles = ptr(v0e1e2, np.float32)
        inp.triangle_count = t.shape[0]
    rgb = np.zeros((width * height, 3), np.float32)
    reads = np.zeros((width * height, 2), np.int32)
    if lib.ref_render(ctypes.byref(inp), rgb.ctypes.data, reads.ctypes.data) != 0:
        raise RuntimeError("reference render failed")
    return rgb, reads
