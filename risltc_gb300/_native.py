"""ctypes bindings of librisltc_gb300.so (the C ABI declared in include/risltc.h).

The library is built in-tree by risltc_gb300/build.py.  Loading it needs no
GPU; device entry points return RISLTC_ERROR_NO_DEVICE without one.
"""
import ctypes
import os

from . import build as _build

c_float_p = ctypes.POINTER(ctypes.c_float)
c_u32_p = ctypes.POINTER(ctypes.c_uint32)


class PolygonalLight(ctypes.Structure):
    """polygonal_light_t, src/polygonal_light.h:73-99."""
    _fields_ = [
        ("rotation_angles", ctypes.c_float * 3), ("scaling_x", ctypes.c_float),
        ("translation", ctypes.c_float * 3), ("scaling_y", ctypes.c_float),
        ("radiant_flux", ctypes.c_float * 3), ("inv_scaling_x", ctypes.c_float),
        ("surface_radiance", ctypes.c_float * 3), ("inv_scaling_y", ctypes.c_float),
        ("plane", ctypes.c_float * 4), ("vertex_count", ctypes.c_uint32),
        ("texturing_technique", ctypes.c_int32), ("texture_index", ctypes.c_uint32),
        ("padding_0", ctypes.c_uint32), ("rotation", (ctypes.c_float * 4) * 3),
        ("area", ctypes.c_float), ("rcp_area", ctypes.c_float), ("padding_1", ctypes.c_float * 2),
        ("texture_file_path", ctypes.c_char_p), ("vertices_plane_space", c_float_p),
        ("vertices_world_space", c_float_p),
    ]


class NoiseTable(ctypes.Structure):
    """noise_table_t, src/noise_table.h:25-29."""
    _fields_ = [("random_seed", ctypes.c_uint32)]


class LtcConstants(ctypes.Structure):
    """ltc_constants_t, src/ltc_table.h:23-35."""
    _fields_ = [("fresnel_index_factor", ctypes.c_float), ("fresnel_index_summand", ctypes.c_float),
                ("roughness_factor", ctypes.c_float), ("roughness_summand", ctypes.c_float),
                ("inclination_factor", ctypes.c_float), ("inclination_summand", ctypes.c_float),
                ("padding", ctypes.c_float * 2)]


class LtcTable(ctypes.Structure):
    _fields_ = [("roughness_count", ctypes.c_uint32), ("inclination_count", ctypes.c_uint32),
                ("fresnel_count", ctypes.c_uint32), ("padding", ctypes.c_uint32),
                ("texels0", c_float_p), ("texels1", c_float_p), ("constants", LtcConstants)]


class Bvh(ctypes.Structure):
    _fields_ = [("node_count", ctypes.c_uint32), ("triangle_count", ctypes.c_uint32),
                ("depth", ctypes.c_uint32), ("padding", ctypes.c_uint32),
                ("nodes", c_float_p), ("triangles", c_float_p), ("triangle_ids", c_u32_p)]


class Settings(ctypes.Structure):
    _fields_ = [("polygon_sampling_technique", ctypes.c_int32), ("light_sampling", ctypes.c_int32),
                ("mis_heuristic", ctypes.c_int32), ("candidate_count", ctypes.c_uint32),
                ("sample_count", ctypes.c_uint32), ("sample_count_light", ctypes.c_uint32),
                ("mis_visibility_estimate", ctypes.c_float), ("fast_atan", ctypes.c_uint32),
                ("shadows", ctypes.c_uint32), ("numerics", ctypes.c_int32), ("proposal", ctypes.c_int32),
                ("proposal_uniform_fraction", ctypes.c_float), ("tile", ctypes.c_int32)]


class GBuffer(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("planes", ctypes.c_void_p), ("primitive", ctypes.c_void_p)]


class Camera(ctypes.Structure):
    """risltc_camera_t = first_person_camera_t, src/camera.h:29-49."""
    _fields_ = [("position_world_space", ctypes.c_float * 3), ("rotation_z", ctypes.c_float),
                ("rotation_x", ctypes.c_float), ("vertical_fov", ctypes.c_float), ("near_plane", ctypes.c_float),
                ("far_plane", ctypes.c_float), ("speed", ctypes.c_float), ("rotate_camera", ctypes.c_int32),
                ("rotation_x_0", ctypes.c_float), ("rotation_z_0", ctypes.c_float)]


class Heightfield(ctypes.Structure):
    """risltc_heightfield_t."""
    _fields_ = [("camera", ctypes.c_float * 3), ("fov_y", ctypes.c_float), ("wave_count", ctypes.c_uint32),
                ("waves", (ctypes.c_float * 4) * 16), ("material_seed", ctypes.c_uint32),
                ("roughness_min", ctypes.c_float), ("roughness_max", ctypes.c_float),
                ("albedo_min", ctypes.c_float), ("albedo_max", ctypes.c_float), ("fresnel_0", ctypes.c_float)]


class BatchItem(ctypes.Structure):
    """risltc_batch_item_t."""
    _fields_ = [("scene", ctypes.c_void_p), ("gbuffer", GBuffer), ("settings", Settings),
                ("noise", ctypes.POINTER(NoiseTable)), ("animate", ctypes.c_uint32), ("frame_count", ctypes.c_uint32),
                ("out_rgb", ctypes.c_void_p), ("accum", ctypes.c_void_p), ("reservoirs", ctypes.c_void_p)]


class Reservoir(ctypes.Structure):
    _fields_ = [("light_index", ctypes.c_int32), ("w_sum", ctypes.c_float),
                ("sample_value", ctypes.c_float), ("padding", ctypes.c_uint32)]


# Exported symbols and their signatures (every declaration of include/risltc.h).
SIGNATURES = {
    "set_polygonal_light_vertex_count": (ctypes.c_int, [ctypes.POINTER(PolygonalLight), ctypes.c_uint32]),
    "update_polygonal_light": (None, [ctypes.POINTER(PolygonalLight)]),
    "duplicate_polygonal_light": (PolygonalLight, [ctypes.POINTER(PolygonalLight)]),
    "destroy_polygonal_light": (None, [ctypes.POINTER(PolygonalLight)]),
    "set_noise_constants": (None, [c_u32_p, c_u32_p, c_u32_p, ctypes.POINTER(NoiseTable), ctypes.c_uint32]),
    "risltc_wang_random_number": (ctypes.c_uint32, [ctypes.c_uint32]),
    "risltc_write_lights": (ctypes.c_int, [c_float_p, ctypes.POINTER(PolygonalLight), ctypes.c_uint32, ctypes.c_uint32]),
    "risltc_max_light_vertex_count": (ctypes.c_uint32, [ctypes.POINTER(PolygonalLight), ctypes.c_uint32]),
    "risltc_ltc_table_from_fit": (ctypes.c_int, [ctypes.POINTER(LtcTable), c_float_p, ctypes.c_uint32,
                                                 ctypes.c_uint32, ctypes.c_int]),
    "risltc_load_ltc_table": (ctypes.c_int, [ctypes.POINTER(LtcTable), ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int]),
    "risltc_ltc_table_synthetic": (ctypes.c_int, [ctypes.POINTER(LtcTable), ctypes.c_uint64, ctypes.c_uint32,
                                                  ctypes.c_uint32]),
    "risltc_ltc_table_destroy": (None, [ctypes.POINTER(LtcTable)]),
    "risltc_bvh_build": (ctypes.c_int, [ctypes.POINTER(Bvh), c_float_p, ctypes.c_uint32, ctypes.c_uint32]),
    "risltc_bvh_destroy": (None, [ctypes.POINTER(Bvh)]),
    "risltc_quick_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Camera),
                                         ctypes.POINTER(ctypes.POINTER(PolygonalLight)), c_u32_p]),
    "risltc_quick_save": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Camera), ctypes.POINTER(PolygonalLight),
                                         ctypes.c_uint32]),
    "risltc_destroy_lights": (None, [ctypes.POINTER(PolygonalLight), ctypes.c_uint32]),
    "risltc_cluster_lights": (ctypes.c_int, [c_float_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                             ctypes.c_uint32, c_u32_p, c_u32_p]),
    "risltc_cluster_summaries": (ctypes.c_int, [c_float_p, ctypes.c_uint32, ctypes.c_uint32, c_u32_p,
                                                ctypes.c_uint32, c_float_p, c_float_p]),
    "risltc_model_parameter_count": (ctypes.c_uint32, [ctypes.c_uint32]),
    "risltc_model_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "risltc_model_destroy": (None, [ctypes.c_void_p]),
    "risltc_model_set_params": (ctypes.c_int, [ctypes.c_void_p, c_float_p]),
    "risltc_model_get_params": (ctypes.c_int, [ctypes.c_void_p, c_float_p]),
    "risltc_model_set_input_transform": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_float]),
    "risltc_model_set_training": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint32]),
    "risltc_model_set_target_mix": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float]),
    "risltc_model_set_training_flags": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32]),
    "risltc_model_get_gradient": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_int]),
    "risltc_model_apply_update": (ctypes.c_int, [ctypes.c_void_p]),
    "risltc_model_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(GBuffer), ctypes.c_void_p,
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "risltc_scene_set_model": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "risltc_model_logits": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(GBuffer), ctypes.c_void_p]),
    "risltc_gbuffer_heightfield": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Heightfield), ctypes.c_uint32,
                                                  ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]),
    "risltc_default_settings": (None, [ctypes.POINTER(Settings)]),
    "risltc_ctx_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_void_p]),
    "risltc_ctx_destroy": (None, [ctypes.c_void_p]),
    "risltc_ctx_reserve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]),
    "risltc_scene_create": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_uint32, ctypes.c_uint32,
                                           ctypes.POINTER(LtcTable), c_float_p, ctypes.c_uint32,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "risltc_scene_destroy": (None, [ctypes.c_void_p]),
    "risltc_scene_set_clusters": (ctypes.c_int, [ctypes.c_void_p, c_u32_p, ctypes.c_uint32]),
    "risltc_shade": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(GBuffer),
                                    ctypes.POINTER(Settings), ctypes.POINTER(NoiseTable), ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "risltc_shade_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchItem), ctypes.c_uint32]),
    "risltc_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(GBuffer),
                                       ctypes.POINTER(Settings), ctypes.POINTER(NoiseTable), ctypes.c_uint32,
                                       ctypes.c_uint32, c_float_p]),
    "risltc_autotune_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchItem), ctypes.c_uint32,
                                             ctypes.c_uint32, c_float_p]),
    "risltc_shade_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                         c_float_p, c_u32_p, ctypes.POINTER(Settings), ctypes.POINTER(NoiseTable),
                                         ctypes.c_uint32, ctypes.c_uint32, c_float_p]),
    "risltc_shade_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(GBuffer), ctypes.POINTER(Settings),
                                            ctypes.POINTER(NoiseTable), ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "risltc_trace_shadow": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                           ctypes.c_void_p]),
    "risltc_ctx_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p, c_u32_p]),
    "risltc_ctx_launch_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "risltc_ctx_ray_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]),
    "risltc_ctx_check": (ctypes.c_int, [ctypes.c_void_p]),
    "risltc_ctx_inject_fault": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32]),
    "risltc_status_string": (ctypes.c_char_p, [ctypes.c_int]),
}

_lib = None


def load(build_if_missing=True):
    """Loads (building first if needed) and returns the product library."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError("librisltc_gb300.so is not built; run risltc_gb300/build.py")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class RisltcError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = load().risltc_status_string(status).decode()
        super().__init__("%s: %s (status %d)" % (what, msg, status) if what else "%s (status %d)" % (msg, status))


def check(status, what=""):
    if status != 0:
        raise RisltcError(status, what)
