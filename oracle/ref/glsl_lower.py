"""Lower the reference renderer's shading-pass GLSL to C++ source text.

Test infrastructure (builds the pinning reference under oracle/_ref); nothing
in the product imports this module.

The reference's per-pixel shading path is GLSL (src/shaders/shading_pass.frag.glsl
and its includes).  To run *that code itself* on the CPU, this module reads the
files where they lie, applies purely mechanical rewrites, and returns C++ text
that is piped straight into g++ (nothing is written to disk):

  * #include "x.glsl" is inlined (once per file); of the related-work
    sampler library (polygon_sampling_related_work.glsl) only the two
    functions of the SAMPLE_POLYGON_AREA_TURK branch (sample_area_polygon_turk
    and get_area_sample_density) are kept, after the polygon_sampling.glsl it
    includes (its solid-angle samplers and cubic solver are not on the path);
  * comments, #version and #extension lines are dropped;
  * parameter qualifiers: `inout T x` / `out T x` become `T& x`, `in T x`
    becomes `T x`, array parameters keep their (pointer) form;
  * layout(...) qualifiers are dropped, uniform/buffer blocks become plain
    globals, global `in`/`out`/`uniform` qualifiers are dropped;
  * the light buffer becomes GlslLightArray<polygonal_light_t> (records reads);
  * the mesh-decoding get_shading_data() is renamed away; the harness supplies
    a G-buffer read with the same signature;
  * main() becomes shading_pass_main(); the hard-coded candidate count
    `int m = 32;` (shading_pass.frag.glsl:726) becomes RISLTC_REF_M;
  * vector constructors whose arguments draw noise (get_noise_2,
    noise_utility.glsl:87-89) use brace initialisation so the two draws are
    evaluated left to right, as GLSL specifies for function arguments.
"""
import os
import re

INCLUDE_RE = re.compile(r'^\s*#include\s+"([^"]+)"\s*$', re.M)


AREA_TURK_FUNCTIONS = ("vec3 sample_area_polygon_turk(", "float get_area_sample_density(")


def _function_text(text, signature_start):
    """The full definition of the function whose signature starts with
    signature_start (up to its matching closing brace)."""
    i = text.index(signature_start)
    j = text.index("{", i)
    depth = 0
    for k in range(j, len(text)):
        depth += {"{": 1, "}": -1}.get(text[k], 0)
        if depth == 0:
            return text[i:k + 1] + "\n"
    raise ValueError("unbalanced braces after " + signature_start)


def _inline(path, shader_dir, seen):
    name = os.path.basename(path)
    if name == "polygon_sampling_related_work.glsl":
        if name in seen:
            return ""
        seen.add(name)
        with open(path, "r") as f:
            related = _strip_comments(f.read())
        base = _inline(os.path.join(shader_dir, "polygon_sampling.glsl"), shader_dir, seen)
        return base + "\n" + "".join(_function_text(related, sig) for sig in AREA_TURK_FUNCTIONS)
    if name in seen:
        return ""
    seen.add(name)
    with open(path, "r") as f:
        text = f.read()

    def repl(m):
        return _inline(os.path.join(shader_dir, m.group(1)), shader_dir, seen)

    return INCLUDE_RE.sub(repl, text)


def _strip_comments(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def _brace_noise_ctors(text):
    """Rewrite vecN( ... ) to vecN{ ... } when the arguments call get_noise_gen."""
    out = []
    i = 0
    pat = re.compile(r"\b(vec[234])\(")
    while True:
        m = pat.search(text, i)
        if not m:
            out.append(text[i:])
            break
        start = m.end() - 1
        depth = 0
        j = start
        while j < len(text):
            if text[j] == "(":
                depth += 1
            elif text[j] == ")":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        args = text[start + 1:j]
        out.append(text[i:m.start()])
        if "get_noise_gen" in args:
            out.append(m.group(1) + "{" + args + "}")
        else:
            out.append(text[m.start():j + 1])
        i = j + 1
    return "".join(out)


def lower(shader_dir, entry="shading_pass.frag.glsl"):
    text = _inline(os.path.join(shader_dir, entry), shader_dir, set())
    text = _strip_comments(text)
    text = re.sub(r"^\s*#(version|extension)[^\n]*$", "", text, flags=re.M)
    # Parameter qualifiers (only directly after '(' or ',').
    param = re.compile(r"([(,]\s*)(?:const\s+)?(inout|out|in)\s+(\w+)\s+(\w+)(\s*\[[^\]]*\])?")

    def param_repl(m):
        lead, qual, typ, name, arr = m.groups()
        if arr:
            return f"{lead}{typ} {name}{arr}"
        if qual == "in":
            return f"{lead}{typ} {name}"
        return f"{lead}{typ}& {name}"

    text = param.sub(param_repl, text)
    text = re.sub(r"\blayout\s*\([^)]*\)\s*", "", text)
    text = re.sub(r"\b(?:uniform|buffer)\s+\w+\s*\{([^{}]*)\}\s*;", r"\1", text)
    text = re.sub(r"\buniform\s+", "", text)
    text = re.sub(r"^(\s*)(?:in|out)\s+(?=\w+\s+\w+\s*;)", r"\1", text, flags=re.M)
    text = re.sub(r"polygonal_light_t\s+g_polygonal_lights\s*\[\s*POLYGONAL_LIGHT_ARRAY_SIZE\s*\]\s*;",
                  "GlslLightArray<polygonal_light_t> g_polygonal_lights;", text)
    text = text.replace("shading_data_t get_shading_data(",
                        "shading_data_t get_shading_data_from_mesh_unused(")
    text = re.sub(r"\bvoid\s+main\s*\(\s*\)",
                  "shading_data_t get_shading_data(ivec2 pixel, int primitive_index, vec3 ray_direction);\n"
                  "void shading_pass_main()", text)
    text, n = re.subn(r"\bint\s+m\s*=\s*32\s*;", "int m = RISLTC_REF_M;", text)
    if n != 1:
        raise RuntimeError("candidate-count literal not found in the shading pass")
    return _brace_noise_ctors(text)


if __name__ == "__main__":
    import sys
    sys.stdout.write(lower(sys.argv[1]))
