"""Generates the golden fixtures under tests/golden/ from the reference itself.

Runs only where the reference sources are present, in the directory named by
the environment variable RISLTC_REFERENCE_DIR (no default):
the reference's shading pass (src/shaders/shading_pass.frag.glsl and its
includes, lowered to C++ by oracle/ref/glsl_lower.py), its clip_polygon, and
its plain-C light model (src/polygonal_light.c) are compiled and executed on
small seeded scenes; inputs and outputs are saved so that the tests (here and
on the GPU machine, where the reference is absent) can compare against them.

Usage: python tests/golden/make_golden.py
"""
import ctypes
import itertools
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle", "ref"))

from risltc_gb300 import _native, scenes  # noqa: E402
import build_ref  # noqa: E402
import ref_runner  # noqa: E402


def reference_light_lib():
    lib = ctypes.CDLL(build_ref.build_ref_host())
    lib.set_polygonal_light_vertex_count.argtypes = [ctypes.POINTER(_native.PolygonalLight), ctypes.c_uint32]
    lib.update_polygonal_light.argtypes = [ctypes.POINTER(_native.PolygonalLight)]
    lib.destroy_polygonal_light.argtypes = [ctypes.POINTER(_native.PolygonalLight)]
    lib.ref_wang_random_number.restype = ctypes.c_uint32
    lib.ref_wang_random_number.argtypes = [ctypes.c_uint32]
    return lib


def noise_numbers(lib, frame):
    """set_noise_constants with animate on (src/noise_table.c:24-28)."""
    return [int(lib.ref_wang_random_number(frame * 4 + i)) for i in range(4)]


CONFIGS = {
    # name: (scene, shader specialisation, frame)
    "quads_m8": ("quads", {"m": 8}, 0),
    "quads_m32": ("quads", {"m": 32}, 1),
    "hf_ltc_cp_m16": ("hf", {"m": 16}, 0),
    "hf_psa_ris_m8": ("hf", {"m": 8, "technique": "projected_solid_angle"}, 0),
    "hf_uniform_psa": ("hf", {"light_sampling": "uniform", "technique": "projected_solid_angle"}, 1),
    "hf_uniform_ltc_cp": ("hf", {"light_sampling": "uniform", "technique": "ltc_cp"}, 0),
    "hf_balance": ("hf", {"m": 8, "mis": "balance"}, 0),
    "hf_power": ("hf", {"m": 8, "mis": "power"}, 0),
    "hf_weighted": ("hf", {"m": 8, "mis": "weighted"}, 0),
    "hf_optimal": ("hf", {"m": 8, "mis": "optimal"}, 0),
    "hf_sc2_ls2": ("hf", {"m": 8, "sample_count": 2, "light_samples": 2}, 0),
    "hf_fast_atan": ("hf", {"m": 8, "fast_atan": 1}, 0),
    "hf_psa_biased": ("hf", {"light_sampling": "uniform", "technique": "projected_solid_angle_biased"}, 0),
    "tris_m8": ("tris", {"m": 8}, 2),
    "octagons_m8": ("oct", {"m": 8}, 0),
    "hf_area_turk_m8": ("hf", {"m": 8, "technique": "area_turk"}, 0),
    "hf_uniform_area_turk": ("hf", {"light_sampling": "uniform", "technique": "area_turk"}, 1),
}


def make_scenes(light_lib):
    out = {
        "quads": scenes.plane_of_quads(32, 32, light_count=64, seed=0, light_lib=light_lib),
        "hf": scenes.heightfield(48, 27, light_count=40, triangle_count=300, seed=1, vertex_counts=(3, 7),
                                 light_lib=light_lib),
        "tris": scenes.heightfield(40, 24, light_count=30, triangle_count=0, seed=2, vertex_counts=(3, 3),
                                   light_lib=light_lib),
        "oct": scenes.heightfield(32, 18, light_count=24, triangle_count=100, seed=3, vertex_counts=(6, 8),
                                  light_lib=light_lib),
    }
    return out


def clip_table():
    """The reference's clip_polygon on every sign pattern of 3..7-gons."""
    so = build_ref.build_ref({"maxv": 7})
    lib = ctypes.CDLL(so)
    clip = lib._Z12clip_polygonjP4vec3
    clip.restype = ctypes.c_uint
    clip.argtypes = [ctypes.c_uint, ctypes.c_void_p]
    maxp = 8
    rng = np.random.default_rng(7)
    inputs, outputs, counts, ns = [], [], [], []
    for n in range(3, 8):
        for bits in itertools.product([0, 1], repeat=n):
            v = np.zeros((maxp, 3), np.float32)
            v[:, :2] = rng.uniform(-2.0, 2.0, (maxp, 2))
            for i in range(maxp):
                mag = rng.uniform(0.1, 1.5)
                v[i, 2] = mag if (i < n and bits[i]) else -mag
            buf = v.copy()
            vc = clip(n, buf.ctypes.data)
            inputs.append(v)
            outputs.append(buf)
            counts.append(vc)
            ns.append(n)
    return {"n": np.array(ns, np.int32), "inputs": np.array(inputs), "outputs": np.array(outputs),
            "vc": np.array(counts, np.int32), "max_polygon_vertex_count": np.int32(maxp)}


def main():
    if not build_ref.reference_available():
        raise SystemExit("reference sources not found; fixtures can only be regenerated next to them")
    light_lib = reference_light_lib()
    manifest = {"wang": {str(s): int(light_lib.ref_wang_random_number(s)) for s in (0, 1, 2, 3, 7, 12345, 2**31)},
                "scenes": {}, "configs": {}}
    sc = make_scenes(light_lib)
    ltc0, ltc1, consts = sc["quads"].ltc0, sc["quads"].ltc1, sc["quads"].ltc_constants
    np.savez_compressed(os.path.join(HERE, "ltc_synthetic_seed0_64.npz"), ltc0=ltc0, ltc1=ltc1, constants=consts)
    for name, s in sc.items():
        np.savez_compressed(os.path.join(HERE, "scene_%s.npz" % name), gbuffer=s.gbuffer,
                            primitive=(s.primitive if s.primitive is not None else np.zeros(0, np.uint32)),
                            lights=s.lights, triangles=s.triangles)
        manifest["scenes"][name] = {"width": s.width, "height": s.height, "max_vertex_count": s.max_vertex_count,
                                    "min_vertex_count": int(min(len(x.plane_vertices) for x in s.light_specs)),
                                    "has_primitive": s.primitive is not None}
    outputs = {}
    for cname, (sname, cfg, frame) in CONFIGS.items():
        s = sc[sname]
        meta = manifest["scenes"][sname]
        rn = noise_numbers(light_lib, frame)
        full = dict(cfg, maxv=meta["max_vertex_count"], minv=meta["min_vertex_count"])
        rgb, reads = ref_runner.render(full, s.width, s.height, s.gbuffer, s.lights, ltc0, ltc1, consts, rn,
                                       triangles9=s.triangles, primitive=s.primitive)
        outputs["rgb_" + cname] = rgb
        outputs["reads_" + cname] = reads
        manifest["configs"][cname] = {"scene": sname, "shader": cfg, "random_numbers": rn,
                                      "candidates": int(cfg.get("m", 32))}
        print(cname, "mean", rgb.mean(0))
    np.savez_compressed(os.path.join(HERE, "reference_outputs.npz"), **outputs)
    np.savez_compressed(os.path.join(HERE, "clip_table.npz"), **clip_table())
    rng = np.random.default_rng(11)
    specs = scenes.polygon_specs(rng, 300, (3, 8)) + scenes.quad_specs(rng, 60)
    lights, maxv = scenes.build_lights(specs, light_lib)
    np.savez_compressed(os.path.join(HERE, "light_model.npz"), lights=lights,
                        angles=np.array([s.rotation_angles for s in specs], np.float32),
                        scaling=np.array([s.scaling for s in specs], np.float32),
                        translation=np.array([s.translation for s in specs], np.float32),
                        flux=np.array([s.radiant_flux for s in specs], np.float32),
                        counts=np.array([len(s.plane_vertices) for s in specs], np.int32),
                        plane_vertices=np.concatenate([s.plane_vertices for s in specs]).astype(np.float32))
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
