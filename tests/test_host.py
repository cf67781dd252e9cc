"""Host-side components on the CPU: math kernels, light model, noise, LTC
quantisation, BVH builder and the exported C ABI."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import golden_data as gd

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from risltc_gb300 import _native
    return _native.load()


def test_library_exports_every_declared_function(lib):
    names = set()
    for header in ("risltc.h",):
        text = open(os.path.join(REPO, "include", header)).read()
        names |= set(re.findall(r"EXTERN_C\s+[\w\s\*]+?\b(\w+)\s*\(", text))
    assert len(names) >= 24
    for n in sorted(names):
        assert hasattr(lib, n), n


NULL_ARGUMENT_CHECK = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
from risltc_gb300 import _native as n
lib = n.load(build_if_missing=False)
# The reference's own light and noise functions dereference their arguments
# as the reference does; every function of this library checks them.
reference_api = {"set_polygonal_light_vertex_count", "update_polygonal_light", "duplicate_polygonal_light",
                 "destroy_polygonal_light", "set_noise_constants"}
checked = 0
for name, (res, args) in sorted(n.SIGNATURES.items()):
    if name in reference_api:
        continue
    for fill in (0, 1):
        vals = [fill if a in (ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64) else float(fill)
                if a is ctypes.c_float else None for a in args]
        r = getattr(lib, name)(*vals)
        if res is ctypes.c_int:
            assert r == 1, (name, fill, r)  # RISLTC_ERROR_INVALID_ARGUMENT
            checked += 1
assert lib.risltc_max_light_vertex_count(None, 5) == 3
print(checked)
"""


def test_entry_points_reject_null_handles_and_arrays(lib):
    """Every status-returning entry point of this library answers null
    handles and arrays (with zero and non-zero counts) with
    RISLTC_ERROR_INVALID_ARGUMENT before it touches a device, and the
    functions without a status (destroy, default settings) accept null.
    Run in a child process, so that a null dereference fails the test
    instead of ending the test run."""
    out = subprocess.run([os.sys.executable, "-c", NULL_ARGUMENT_CHECK, REPO], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    from risltc_gb300 import _native
    statuses = [k for k, (res, _) in _native.SIGNATURES.items() if res is ctypes.c_int and k.startswith("risltc_")]
    assert len(statuses) >= 35 and int(out.stdout.strip()) == 2 * len(statuses)


def test_math_kernels_against_libm(tmp_path):
    src = tmp_path / "m.c"
    src.write_text('#include "risltc_math.h"\n'
                   "void eval(const float* x, int n, float* a, float* c, float* s, float* co) {\n"
                   "  for (int i = 0; i < n; ++i) { a[i] = rl_atanf(x[i]); c[i] = rl_acosf(x[i] > 1 ? 1 : "
                   "(x[i] < -1 ? -1 : x[i]));\n"
                   "    rl_sincosf(x[i], &s[i], &co[i]); } }\n")
    so = tmp_path / "m.so"
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-ffp-contract=off", "-I", os.path.join(REPO, "include"),
                    str(src), "-o", str(so)], check=True)
    m = ctypes.CDLL(str(so))
    x = np.concatenate([np.linspace(-20, 20, 400001), np.linspace(-1, 1, 100001), [0.0, -0.0, 1e-30, 1e30]])
    x = x.astype(np.float32)
    out = [np.zeros_like(x) for _ in range(4)]
    m.eval(x.ctypes.data, len(x), *[o.ctypes.data for o in out])
    xd = x.astype(np.float64)

    def ulp_err(got, want):
        return np.abs(got.astype(np.float64) - want) / np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)

    assert ulp_err(out[0], np.arctan(xd)).max() <= 2.0
    xc = np.clip(xd, -1, 1)
    # acos near 1 has a tiny result; bound the absolute error there.
    assert (np.abs(out[1] - np.arccos(xc)) <= 4 * np.spacing(np.float32(np.pi))).all()
    small = np.abs(xd) <= 16.0
    assert np.abs(out[2][small] - np.sin(xd[small])).max() <= 2.5e-7
    assert np.abs(out[3][small] - np.cos(xd[small])).max() <= 2.5e-7


def test_light_model_matches_reference_polygonal_light_c(lib):
    from risltc_gb300 import scenes
    d = np.load(os.path.join(gd.GOLDEN, "light_model.npz"))
    specs, offset = [], 0
    for i, n in enumerate(d["counts"]):
        specs.append(scenes.LightSpec(tuple(d["angles"][i]), tuple(d["scaling"][i]), tuple(d["translation"][i]),
                                      tuple(d["flux"][i]), d["plane_vertices"][offset:offset + n]))
        offset += n
    lights, _ = scenes.build_lights(specs)
    assert np.array_equal(lights.view(np.uint32), d["lights"].view(np.uint32))


def test_write_lights_and_vertex_count_behaviour(lib):
    from risltc_gb300 import _native
    light = _native.PolygonalLight()
    # The reference reports 0 even when the count changes (polygonal_light.c:39-40).
    assert lib.set_polygonal_light_vertex_count(ctypes.byref(light), 5) == 0
    assert light.vertex_count == 5
    for v in range(5):
        light.vertices_plane_space[4 * v] = np.cos(2 * np.pi * v / 5)
        light.vertices_plane_space[4 * v + 1] = np.sin(2 * np.pi * v / 5)
    light.scaling_x = light.scaling_y = 2.0
    lib.update_polygonal_light(ctypes.byref(light))
    area = 0.5 * 5 * np.sin(2 * np.pi / 5) * 4.0
    assert abs(light.area - area) < 1e-5 * area
    copy = lib.duplicate_polygonal_light(ctypes.byref(light))
    assert copy.vertex_count == 5 and copy.vertices_plane_space[4] == light.vertices_plane_space[4]
    buf = np.zeros((1, 12 + 4 * 8), np.float32)
    assert lib.risltc_write_lights(buf.ctypes.data_as(_native.c_float_p), ctypes.byref(light), 1, 8) == 0
    assert buf[0, 8:9].view(np.uint32)[0] == 5
    assert np.array_equal(buf[0, 12 + 4 * 5:15 + 4 * 5], buf[0, 12:15])  # slot 5 repeats vertex 0
    assert lib.risltc_write_lights(buf.ctypes.data_as(_native.c_float_p), ctypes.byref(light), 1, 4) == 2
    assert lib.risltc_write_lights(buf.ctypes.data_as(_native.c_float_p), ctypes.byref(light), 1, 9) == 1
    lib.destroy_polygonal_light(ctypes.byref(copy))
    lib.destroy_polygonal_light(ctypes.byref(light))
    assert light.vertex_count == 0 and not light.vertices_plane_space


def test_noise_constants_match_reference(lib):
    from risltc_gb300 import _native
    for seed, want in gd.manifest()["wang"].items():
        assert lib.risltc_wang_random_number(int(seed)) == want
    rn = (ctypes.c_uint32 * 4)()
    nt = _native.NoiseTable(3)
    lib.set_noise_constants(None, None, rn, ctypes.byref(nt), 1)
    assert list(rn) == [lib.risltc_wang_random_number(12 + i) for i in range(4)] and nt.random_seed == 4
    lib.set_noise_constants(None, None, rn, ctypes.byref(nt), 0)
    assert list(rn) == [0, 0x123456, 2 * 0x123456, 3 * 0x123456] and nt.random_seed == 5


def quantize_reference(d, unorm16):
    """numpy restatement of load_ltc_table's loop (src/ltc_table.c:82-116)."""
    d = d.astype(np.float32)
    inv = np.zeros(d.shape[:-1] + (3, 3), np.float32)
    inv[..., 0, 0] = d[..., 2]
    inv[..., 0, 2] = -d[..., 1] * d[..., 2]
    inv[..., 1, 1] = d[..., 0] - d[..., 1] * d[..., 3]
    inv[..., 2, 0] = -d[..., 2] * d[..., 3]
    inv[..., 2, 2] = d[..., 0] * d[..., 2]
    mx = np.max(np.abs(inv), axis=(-1, -2), keepdims=True)
    inv = inv / mx
    vals = np.stack([inv[..., 0, 0], -inv[..., 0, 2], inv[..., 1, 1], inv[..., 2, 0], inv[..., 2, 2], d[..., 4]], -1)
    vals = np.clip(vals, 0.0, 1.0)
    if unorm16:
        vals = np.floor(vals * np.float32(65535.0) + np.float32(0.5)).astype(np.uint16).astype(np.float32) / \
            np.float32(65535.0)
    return vals


@pytest.mark.parametrize("unorm16", [0, 1])
def test_ltc_table_from_fit_quantisation(lib, tmp_path, unorm16):
    from risltc_gb300 import _native
    rng = np.random.default_rng(4)
    res, layers = 8, 3
    fit = np.empty((layers, res, res, 5), np.float32)
    fit[..., 0] = rng.uniform(0.2, 3.0, fit.shape[:-1])
    fit[..., 1] = rng.uniform(0.0, 0.5, fit.shape[:-1])
    fit[..., 2] = rng.uniform(0.2, 3.0, fit.shape[:-1])
    fit[..., 3] = rng.uniform(-0.5, 0.0, fit.shape[:-1])
    fit[..., 4] = rng.uniform(0.0, 1.0, fit.shape[:-1])
    t = _native.LtcTable()
    assert lib.risltc_ltc_table_from_fit(ctypes.byref(t), fit.ctypes.data_as(_native.c_float_p), res, layers,
                                         unorm16) == 0
    n = res * res * layers
    got0 = np.ctypeslib.as_array(t.texels0, shape=(4 * n,)).copy().reshape(layers, res, res, 4)
    got1 = np.ctypeslib.as_array(t.texels1, shape=(2 * n,)).copy().reshape(layers, res, res, 2)
    want = quantize_reference(fit, unorm16)
    assert np.allclose(got0, want[..., :4], atol=1e-7) and np.allclose(got1, want[..., 4:], atol=1e-7)
    c = t.constants
    assert c.fresnel_index_factor == layers - 1 and abs(c.roughness_factor - (res - 1) / res) < 1e-7
    assert abs(c.inclination_summand - 0.5 / res) < 1e-7
    lib.risltc_ltc_table_destroy(ctypes.byref(t))
    # The same records through fit<i>.dat files (uint64 resolution header).
    for i in range(layers):
        with open(tmp_path / ("fit%d.dat" % i), "wb") as f:
            f.write(np.uint64(res).tobytes())
            f.write(fit[i].tobytes())
    t2 = _native.LtcTable()
    assert lib.risltc_load_ltc_table(ctypes.byref(t2), str(tmp_path).encode(), layers, unorm16) == 0
    assert np.array_equal(np.ctypeslib.as_array(t2.texels0, shape=(4 * n,)), got0.ravel())
    lib.risltc_ltc_table_destroy(ctypes.byref(t2))
    assert lib.risltc_load_ltc_table(ctypes.byref(t2), b"/nonexistent", 1, 0) == 8


def test_synthetic_ltc_table_is_valid():
    from risltc_gb300 import scenes
    l0, l1, k = scenes.synthetic_ltc(0, 64)
    assert l0.shape == (1, 64, 64, 4) and l1.shape == (1, 64, 64, 2)
    assert (l0 >= 0).all() and (l0 <= 1).all() and (l1 >= 0).all() and (l1 <= 1).all()
    det2 = l0[..., 0] * l1[..., 0] + l0[..., 1] * l0[..., 3]
    assert (det2 > 0).all() and (l0[..., 2] > 0).all()
    assert np.abs(np.diff(l0, axis=2)).max() < 0.2  # smooth in roughness
    assert np.array_equal(l0, gd.ltc()[0])


def test_bvh_invariants():
    """Nested boxes; every reference in exactly one leaf; every triangle
    referenced at least once (large ones cut into pieces, at most three
    references per triangle in all); and conservative leaves: points all over
    each triangle lie in the box of a leaf that references it, so a ray that
    hits a triangle reaches a leaf that tests it."""
    from risltc_gb300 import api, scenes
    rng = np.random.default_rng(0)
    tris = scenes.random_triangles(rng, 5000)
    nodes, reordered, ids, depth = api.build_bvh(tris)
    assert set(ids.tolist()) == set(range(5000))
    assert 5000 < len(ids) <= 3 * 5000
    assert depth <= 60
    words = nodes.view(np.int32)
    v0 = tris.reshape(-1, 3, 3)[ids]
    assert np.array_equal(reordered[:, 0:3], v0[:, 0])
    assert np.array_equal(reordered[:, 4:7], v0[:, 1] - v0[:, 0])
    covered = np.zeros(len(ids), int)
    leaf_boxes = {}

    def visit(i, lo, hi):
        n = nodes[i]
        assert (n[0:3] <= n[4:7]).all()
        assert (lo <= n[0:3] + 1e-6).all() and (n[4:7] <= hi + 1e-6).all()
        first, count = words[i, 3], words[i, 7]
        if count == 0:
            visit(first, n[0:3], n[4:7])
            visit(first + 1, n[0:3], n[4:7])
        else:
            for k in range(first, first + count):
                covered[k] += 1
                leaf_boxes.setdefault(int(ids[k]), []).append((n[0:3], n[4:7]))

    import sys
    sys.setrecursionlimit(10000)
    visit(0, nodes[0, 0:3], nodes[0, 4:7])
    assert (covered == 1).all()
    t = tris.reshape(-1, 3, 3).astype(np.float64)
    bary = np.concatenate([np.eye(3), [[0.5, 0.5, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [1 / 3, 1 / 3, 1 / 3]],
                           rng.dirichlet([1, 1, 1], 24)])
    for tri in range(5000):
        pts = (bary @ t[tri]).astype(np.float32)
        inside = np.zeros(len(pts), bool)
        for lo, hi in leaf_boxes[tri]:
            inside |= ((pts >= lo) & (pts <= hi)).all(axis=1)
        assert inside.all(), tri
    assert api.build_bvh(np.zeros((0, 9), np.float32))[0].shape == (0, 8)


@pytest.mark.parametrize("kind", ["small", "large", "mixed"])
def test_bvh_shadow_answers_equal_brute_force(kind):
    """The oracle's frame with shadow rays traced through the product's BVH
    (split-clipped references) equals the same frame with every triangle
    tested, pixel for pixel: small occluders, large ones (cut into pieces),
    and a mix with degenerate and axis-aligned triangles."""
    import oracle
    from risltc_gb300 import api, scenes
    hs = scenes.heightfield(96, 54, light_count=24, triangle_count=0, seed=3)
    rng = np.random.default_rng(11)
    small = scenes.random_triangles(rng, 1500)
    large = scenes.random_triangles(rng, 300, edge=(1.0, 4.0))
    if kind == "small":
        tris = small
    elif kind == "large":
        tris = large
    else:
        flat = scenes.random_triangles(rng, 200, edge=(0.5, 3.0)).reshape(-1, 3, 3)
        flat[:, :, 2] = 1.0  # axis-aligned: all in the plane z = 1
        degenerate = scenes.random_triangles(rng, 50).reshape(-1, 3, 3)
        degenerate[:, 2] = degenerate[:, 1]
        tris = np.concatenate([small.reshape(-1, 9), large.reshape(-1, 9), flat.reshape(-1, 9),
                               degenerate.reshape(-1, 9)]).astype(np.float32)
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    nodes, refs, ids, _ = api.build_bvh(tris)
    if kind != "small":
        assert len(ids) > len(tris)
    st = oracle.make_settings(candidates=8)
    rn = api.noise_constants(5)[0]
    through = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants, refs, nodes)
    brute = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants,
                               oracle.triangles_v0e1e2(tris))
    a, _, _ = oracle.render(through, st, hs.gbuffer, hs.width, hs.height, rn, reservoirs=False)
    b, _, _ = oracle.render(brute, st, hs.gbuffer, hs.width, hs.height, rn, reservoirs=False)
    assert np.array_equal(a, b)
    unshadowed = oracle.OracleScene(hs.lights, hs.max_vertex_count, hs.ltc0, hs.ltc1, hs.ltc_constants)
    c, _, _ = oracle.render(unshadowed, st, hs.gbuffer, hs.width, hs.height, rn, reservoirs=False)
    assert not np.array_equal(a, c)  # the occluders do shadow the frame


def test_transcendental_coefficients_meet_their_error_bounds():
    """include/risltc_math.h's polynomial coefficients, evaluated in FP32 as
    the header does, stay within the bounds it states (the fit script's own
    check; it also refits them by the header's method)."""
    import subprocess
    import sys
    script = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "risltc_gb300", "csrc",
                          "fit_math_coeffs.py")
    out = subprocess.run([sys.executable, script], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
