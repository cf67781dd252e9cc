"""The C ABI from its two kinds of callers, compiled here from committed sources.

* tests/c/host_frame.c: a C99 host program that includes only
  include/risltc.h and links librisltc_gb300.so, filling polygonal_light_t
  records through the reference's own light API (polygonal_light.h:73-136),
  packing them with risltc_write_lights (write_lights, main.c:456-490) and
  shading one frame with risltc_shade_host.  On the GPU its image must equal
  the oracle's frame of the inputs it wrote, bit for bit.
* tests/cuda/device_routines.cu: a caller's own kernel composed from the
  GLSL-named routines of include/risltc_device.cuh (clip_polygon,
  calculate_ltc, prepare_/sample_projected_solid_angle_polygon,
  polygon_clipping.glsl:35, polygon_sampling.glsl:523, 545, 772).  On the GPU
  its results must equal the oracle's routines bit for bit.

The compile steps run on the CPU too (gcc -std=c99 -pedantic -Werror; nvcc
for sm_103a); without a GPU the host program must get through its host-side
part and stop at the device with RISLTC_ERROR_NO_DEVICE.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import cuda_available

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NO_DEVICE = 6  # RISLTC_ERROR_NO_DEVICE


def library():
    from risltc_gb300 import build
    return build.build()


def compile_host_frame(out_dir):
    lib = library()
    exe = os.path.join(out_dir, "host_frame")
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "c", "host_frame.c"), "-L", os.path.dirname(lib), "-lrisltc_gb300",
                    "-Wl,-rpath," + os.path.dirname(lib), "-lm", "-o", exe], check=True)
    return exe


def compile_device_routines(out_dir):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    so = os.path.join(out_dir, "libdevice_routines.so")
    subprocess.run([nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "--fmad=false",
                    "-prec-div=true", "-prec-sqrt=true", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                    "-shared", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "cuda", "device_routines.cu"), "-o", so], check=True)
    return so


def read_frame_inputs(d):
    maxv, lights, tris, rn_x, width, height = [int(x) for x in open(os.path.join(d, "meta.txt")).read().split()]
    f32 = lambda name: np.fromfile(os.path.join(d, name), np.float32)  # noqa: E731
    return dict(max_vertex_count=maxv, lights=f32("lights.f32").reshape(lights, 12 + 4 * maxv),
                triangles=f32("triangles.f32").reshape(tris, 9), random_number_x=rn_x, width=width, height=height,
                gbuffer=f32("gbuffer.f32").reshape(17, width * height),
                ltc0=f32("ltc0.f32").reshape(1, 64, 64, 4), ltc1=f32("ltc1.f32").reshape(1, 64, 64, 2),
                constants=f32("ltc_constants.f32"))


def test_host_program_compiles_as_c99_and_runs_its_host_part(tmp_path):
    exe = compile_host_frame(str(tmp_path))
    rc = subprocess.run([exe, str(tmp_path), "48", "32", "20", "100"]).returncode
    assert rc == (0 if cuda_available() else NO_DEVICE)
    f = read_frame_inputs(str(tmp_path))
    n = f["lights"][:, 8].view(np.uint32)
    assert np.all((n >= 3) & (n <= 8)) and f["max_vertex_count"] == n.max()
    # update_polygonal_light gave every light a unit plane normal and a plane
    # through its world-space vertices.
    plane = f["lights"][:, 4:8].astype(np.float64)
    assert np.allclose(np.linalg.norm(plane[:, :3], axis=1), 1.0, atol=1e-5)
    verts = f["lights"][:, 12:].reshape(len(n), -1, 4)[:, :, :3].astype(np.float64)
    assert np.abs(np.einsum("lvk,lk->lv", verts, plane[:, :3]) + plane[:, 3:4]).max() < 1e-4


def test_device_routine_header_compiles_for_sm103a(tmp_path):
    assert os.path.getsize(compile_device_routines(str(tmp_path))) > 0


@pytest.mark.gpu
def test_host_program_frame_equals_oracle(gpu, tmp_path):
    exe = compile_host_frame(str(tmp_path))
    subprocess.run([exe, str(tmp_path), "320", "180", "200", "2000"], check=True)
    f = read_frame_inputs(str(tmp_path))
    image = np.fromfile(os.path.join(str(tmp_path), "image.f32"), np.float32).reshape(-1, 3)
    osc = oracle.OracleScene(f["lights"], f["max_vertex_count"], f["ltc0"], f["ltc1"], f["constants"],
                             oracle.triangles_v0e1e2(f["triangles"]))
    want, _, _ = oracle.render(osc, oracle.make_settings(candidates=32), f["gbuffer"], f["width"], f["height"],
                               f["random_number_x"])
    assert (want.sum(1) > 0).mean() > 0.5
    assert np.array_equal(image, want)


def random_polygons(rng, count):
    """Convex polygons of 3..8 vertices on circles in random planes around
    points of [-1, 1]^2 x [-0.6, 1.4]: many cross z = 0."""
    n = rng.integers(3, 9, count).astype(np.uint32)
    xyz = np.zeros((count, 8, 3), np.float32)
    for c in range(count):
        centre = rng.uniform([-1.0, -1.0, -0.6], [1.0, 1.0, 1.4])
        a = rng.normal(size=3)
        a /= np.linalg.norm(a)
        b = np.cross(a, rng.normal(size=3))
        b /= np.linalg.norm(b)
        radius = rng.uniform(0.1, 0.8)
        angles = np.sort(rng.uniform(0.0, 2 * np.pi, n[c]))
        for j, t in enumerate(angles):
            xyz[c, j] = centre + radius * (np.cos(t) * a + np.sin(t) * b)
    return n, xyz


@pytest.mark.gpu
def test_device_routines_equal_oracle(gpu, tmp_path):
    lib = ctypes.CDLL(compile_device_routines(str(tmp_path)))
    lib.risltc_test_polygon_routines.restype = ctypes.c_int
    rng = np.random.default_rng(7)
    count, samples = 2000, 4
    n, xyz = random_polygons(rng, count)
    rnd = rng.uniform(0.0, 1.0, (count, samples, 2)).astype(np.float32)
    vc = np.zeros(count, np.uint32)
    clipped = np.zeros((count, 9, 3), np.float32)
    ltc = np.zeros(count, np.float32)
    psa = np.zeros(count, np.float32)
    dirs = np.zeros((count, samples, 3), np.float32)
    p = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    assert lib.risltc_test_polygon_routines(count, p(n), p(xyz), samples, p(rnd), p(vc), p(clipped), p(ltc), p(psa),
                                            p(dirs)) == 0
    ol = oracle.load()
    ol.oracle_f32_clip_polygon.restype = ctypes.c_uint32
    ol.oracle_f32_clip_polygon.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int]
    ol.oracle_f32_calculate_ltc.restype = ctypes.c_float
    ol.oracle_f32_calculate_ltc.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
    ol.oracle_f32_psa_sample.restype = ctypes.c_float
    ol.oracle_f32_psa_sample.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
    partial = 0
    for c in range(count):
        buf = np.zeros((9, 3), np.float32)
        buf[:8] = xyz[c]
        want_vc = ol.oracle_f32_clip_polygon(int(n[c]), buf.ctypes.data, 9, 0)
        assert vc[c] == want_vc, c
        if want_vc == 0:
            continue
        partial += int(want_vc != n[c])
        poly = np.ascontiguousarray(buf[:want_vc])
        assert np.array_equal(clipped[c, :want_vc], poly), c
        assert ltc[c] == np.float32(ol.oracle_f32_calculate_ltc(int(want_vc), poly.ctypes.data)), c
        want_dirs = np.zeros((samples, 3), np.float32)
        r = np.ascontiguousarray(rnd[c])
        total = ol.oracle_f32_psa_sample(int(want_vc), poly.ctypes.data, samples, r.ctypes.data,
                                         want_dirs.ctypes.data, None)
        assert psa[c] == np.float32(total) or (np.isnan(psa[c]) and np.isnan(total)), c
        # A sliver left by the clipper can have no projected solid angle; its
        # samples are NaN on both sides.
        assert np.array_equal(dirs[c], want_dirs, equal_nan=True), c
    assert partial > 100  # the clipped cases were exercised
