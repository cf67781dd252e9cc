"""Quicksave files (quick_save / quick_load, src/main.c:45-125; the Blender
exporter's reader and writer, tools/io_export_lights_blender.py:11-112).

The files here are written byte by byte from that layout by this test (no
reference quicksave is distributed with the reference), then read through the
C ABI; the lights must come out bit-identical to the same parameters run
through the light model directly.
"""
import struct

import numpy as np
import pytest

CAMERA = (1.5, -2.0, 3.25, 0.3, -0.7, 1.1, 0.05, 200.0, 2.0, 1, 0.25, -0.5)


def write_quicksave(path, specs, texture_paths, legacy):
    with open(path, "wb") as f:
        # first_person_camera_t: 9 floats, int rotate_camera, 2 floats
        f.write(struct.pack("<9fi2f", *CAMERA))
        f.write(struct.pack("<II", 0, len(specs)))
        for s, tex, old in zip(specs, texture_paths, legacy):
            n = len(s.plane_vertices)
            sy = 0.0 if old else s.scaling[1]
            # rotation_angles, scaling_x, translation, scaling_y, radiant_flux,
            # inv_scaling_x, surface_radiance, inv_scaling_y, plane,
            # vertex_count, texturing_technique
            f.write(struct.pack("<3ff3ff3ff3ff4fII", *s.rotation_angles, s.scaling[0], *s.translation, sy,
                                *s.radiant_flux, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, n, 0))
            if tex is None:
                f.write(struct.pack("<Q", 0))
            else:
                raw = tex.encode("ascii") + b"\0"
                f.write(struct.pack("<Q", len(raw)) + raw)
            f.write(struct.pack("<QQ", 0, 0))
            for px, py in s.plane_vertices:
                f.write(struct.pack("<4f", px, py, 0.0, 0.0))


def light_rows(buf, maxv):
    """(radiance, plane, count, world vertices) of each std140 row."""
    out = []
    for row in buf:
        n = int(row[8:9].view(np.uint32)[0])
        verts = row[12:12 + 4 * n].reshape(n, 4)[:, :3]
        out.append((row[0:3].copy(), row[4:8].copy(), n, verts.copy()))
    return out


def test_quick_load_matches_the_light_model(tmp_path):
    from risltc_gb300 import scenes
    rng = np.random.default_rng(11)
    specs = scenes.polygon_specs(rng, 24, vertex_counts=(3, 8))
    textures = [None] * 24
    textures[3] = "data/textures/lamp_3.png"
    legacy = [False] * 24
    legacy[5] = True
    path = tmp_path / "scene.save"
    write_quicksave(path, specs, textures, legacy)
    camera, buf, maxv = scenes.load_quicksave(path)
    assert list(camera.position_world_space) == [np.float32(v) for v in CAMERA[:3]]
    assert camera.rotate_camera == 1 and np.float32(camera.rotation_z_0) == np.float32(CAMERA[11])
    # A legacy light (scaling_y <= 0) gets scaling_y = scaling_x.
    fixed = [scenes.LightSpec(s.rotation_angles, (s.scaling[0], s.scaling[0]) if old else s.scaling,
                              s.translation, s.radiant_flux, s.plane_vertices) for s, old in zip(specs, legacy)]
    want, want_maxv = scenes.build_lights(fixed)
    assert maxv == want_maxv
    for (r0, p0, n0, v0), (r1, p1, n1, v1) in zip(light_rows(buf, maxv), light_rows(want, want_maxv)):
        assert n0 == n1
        assert np.array_equal(r0, r1) and np.array_equal(p0, p1) and np.array_equal(v0, v1)


def test_quick_save_round_trip(tmp_path):
    from risltc_gb300 import scenes
    rng = np.random.default_rng(12)
    specs = scenes.polygon_specs(rng, 10, vertex_counts=(3, 6))
    src, dst = tmp_path / "a.save", tmp_path / "b.save"
    write_quicksave(src, specs, ["tex_%d.png" % i if i % 4 == 0 else None for i in range(10)], [False] * 10)
    scenes.resave_quicksave(src, dst)
    c0, b0, m0 = scenes.load_quicksave(src)
    c1, b1, m1 = scenes.load_quicksave(dst)
    assert bytes(c0) == bytes(c1) and m0 == m1 and np.array_equal(b0, b1)
    # Same size: fixed part, path, two pointers and vertices per light.
    assert src.stat().st_size == dst.stat().st_size


def test_quick_load_errors(tmp_path):
    from risltc_gb300 import scenes, RisltcError
    with pytest.raises(RisltcError):
        scenes.load_quicksave(tmp_path / "missing.save")
    rng = np.random.default_rng(13)
    specs = scenes.polygon_specs(rng, 4)
    path = tmp_path / "cut.save"
    write_quicksave(path, specs, [None] * 4, [False] * 4)
    data = path.read_bytes()
    path.write_bytes(data[:-10])
    with pytest.raises(RisltcError):
        scenes.load_quicksave(path)
