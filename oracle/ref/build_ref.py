"""Build the pinning reference: the reference renderer's own shading-pass GLSL,
lowered to C++ (glsl_lower.py) and compiled with g++ into oracle/_ref/.

Test infrastructure.  Runs only where the reference sources are present, in
the directory named by the environment variable RISLTC_REFERENCE_DIR (no
default); machines without them never need it, because the reference's
outputs are committed as fixtures under tests/golden/.

Each shader specialisation (the defines of main.c:962-990) is its own shared
library, named by its configuration tag.
"""
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
OUT_DIR = os.path.join(ORACLE, "_ref")
REFERENCE_DIR = os.environ.get("RISLTC_REFERENCE_DIR", "")
SHADER_DIR = os.path.join(REFERENCE_DIR, "src", "shaders") if REFERENCE_DIR else ""

sys.path.insert(0, HERE)
import glsl_lower  # noqa: E402

MIS = ["balance", "power", "weighted", "optimal_clamped", "optimal"]
TECHNIQUES = ["baseline", "area_turk", "projected_solid_angle", "projected_solid_angle_biased", "ltc_cp"]


def reference_available():
    return bool(SHADER_DIR) and os.path.isfile(os.path.join(SHADER_DIR, "shading_pass.frag.glsl"))


def _defines(cfg):
    maxv = int(cfg.get("maxv", 4))
    minv = int(cfg.get("minv", 3))
    ls = int(cfg.get("light_samples", 1))
    sc = int(cfg.get("sample_count", 1))
    mis = cfg.get("mis", "optimal_clamped")
    tech = cfg.get("technique", "ltc_cp")
    uniform = cfg.get("light_sampling", "ris") == "uniform"
    d = {
        "MATERIAL_COUNT": 1,
        "POLYGONAL_LIGHT_COUNT": "g_ref_light_count",
        "POLYGONAL_LIGHT_ARRAY_SIZE": 1,
        "POLYGONAL_LIGHT_COUNT_CLAMPED": 33,
        "LIGHT_SAMPLES": ls,
        "LIGHT_SAMPLES_CLAMPED": min(ls, 33),
        "LIGHT_TEXTURE_COUNT": 1,
        "MIN_POLYGON_VERTEX_COUNT_BEFORE_CLIPPING": minv,
        "MAX_POLYGONAL_LIGHT_VERTEX_COUNT": maxv,
        "MAX_POLYGON_VERTEX_COUNT": maxv + 1,
        "SAMPLE_COUNT": sc,
        "SAMPLE_COUNT_CLAMPED": min(sc, 33),
        "SAMPLE_LIGHT_UNIFORM": int(uniform),
        "SAMPLE_LIGHT_RIS": int(not uniform),
        "USE_FAST_ATAN": int(cfg.get("fast_atan", 0)),
        "ERROR_DISPLAY_DIFFUSE": 0,
        "ERROR_DISPLAY_SPECULAR": 0,
        "ERROR_INDEX": 0,
        "RISLTC_REF_M": int(cfg.get("m", 32)),
    }
    for name in MIS:
        d["MIS_HEURISTIC_" + name.upper()] = int(mis == name)
    d["SAMPLE_POLYGON_BASELINE"] = int(tech == "baseline")
    d["SAMPLE_POLYGON_AREA_TURK"] = int(tech == "area_turk")
    d["SAMPLE_POLYGON_PROJECTED_SOLID_ANGLE"] = int(tech in ("projected_solid_angle", "projected_solid_angle_biased"))
    d["SAMPLE_POLYGON_LTC_CP"] = int(tech == "ltc_cp")
    if tech == "projected_solid_angle_biased":
        d["USE_BIASED_PROJECTED_SOLID_ANGLE_SAMPLING"] = 1
    else:
        d["DONT_USE_BIASED_PROJECTED_SOLID_ANGLE_SAMPLING"] = 1
    return d


def config_tag(cfg):
    items = sorted(_defines(cfg).items())
    return hashlib.sha1(repr(items).encode()).hexdigest()[:12]


def build_ref(cfg, force=False):
    """Compiles one specialisation; returns the path of the shared library."""
    if not reference_available():
        raise FileNotFoundError("reference shaders not found at " + SHADER_DIR)
    os.makedirs(OUT_DIR, exist_ok=True)
    out = os.path.join(OUT_DIR, "ref_shading_pass_%s.so" % config_tag(cfg))
    if os.path.exists(out) and not force:
        return out
    source = ('#include "glsl_shim.hpp"\n#include <vector>\n'
              + glsl_lower.lower(SHADER_DIR)
              + '\n#include "ref_harness.hpp"\n')
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-fsingle-precision-constant", "-Wno-narrowing", "-w",
           "-I", HERE, "-I", os.path.join(REPO, "include")]
    for k, v in _defines(cfg).items():
        cmd.append("-D%s=%s" % (k, v))
    cmd += ["-x", "c++", "-", "-o", out + ".tmp"]
    proc = subprocess.run(cmd, input=source, text=True, capture_output=True)
    if proc.returncode != 0:
        raise RuntimeError("g++ failed on the lowered reference shader:\n" + proc.stderr[-6000:])
    os.replace(out + ".tmp", out)
    return out


def build_ref_host(force=False):
    """Compiles the reference's plain-C light model (src/polygonal_light.c,
    with math_utilities.h and string_utilities.h) from where it lies, plus
    ref_host_harness.c, into oracle/_ref/libref_host.so."""
    src_dir = os.path.join(REFERENCE_DIR, "src")
    if not os.path.isfile(os.path.join(src_dir, "polygonal_light.c")):
        raise FileNotFoundError("reference sources not found at " + src_dir)
    os.makedirs(OUT_DIR, exist_ok=True)
    out = os.path.join(OUT_DIR, "libref_host.so")
    if os.path.exists(out) and not force:
        return out
    cmd = ["gcc", "-std=c99", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-I", src_dir, os.path.join(src_dir, "polygonal_light.c"),
           os.path.join(HERE, "ref_host_harness.c"), "-o", out + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_ref({}, force="--force" in sys.argv))
    print(build_ref_host(force="--force" in sys.argv))
