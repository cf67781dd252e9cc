"""risltc_shade_noalloc: the allocation-free variant of risltc_shade.

Callers that may not allocate device memory while rendering (a plugin inside
a host application that owns the device memory budget, or a frame loop that
must not stall other streams through cudaMalloc/cudaFree) create the scene
once and shade each frame through this entry point.  Its scratch lives in a
static device array of RISLTC_NOALLOC_MAX_PIXEL_FRAMES reservoir records.

This file is collected last, so a run that stops at the first failure has run
every other test before it.  It also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import golden_data as gd

pytestmark = pytest.mark.gpu

MAX_PIXEL_FRAMES = 262144  # RISLTC_NOALLOC_MAX_PIXEL_FRAMES in include/risltc.h
TOO_LARGE = 10             # RISLTC_ERROR_TOO_LARGE
INVALID_ARGUMENT = 1       # RISLTC_ERROR_INVALID_ARGUMENT


def test_noalloc_matches_shade_on_two_calls_in_a_row(gpu):
    import torch
    import risltc_gb300 as rl
    from risltc_gb300 import _native
    lib = _native.load()
    lib.risltc_shade_noalloc.restype = ctypes.c_int
    lib.risltc_shade_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(_native.GBuffer),
                                         ctypes.POINTER(_native.Settings), ctypes.POINTER(_native.NoiseTable),
                                         ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
    c = gd.config("hf_ltc_cp_m16")
    sc = gd.scene(c["scene"])
    l0, l1, k = gd.ltc()
    ctx = rl.Context(0)
    scene = rl.Scene(ctx, sc["lights"], sc["max_vertex_count"], l0, l1, k, sc["triangles"])
    s = rl.settings(candidates=c["candidates"])
    p = sc["width"] * sc["height"]
    g = torch.from_numpy(np.ascontiguousarray(sc["gbuffer"])).cuda()
    prim = torch.from_numpy(sc["primitive"].view(np.int32)).cuda()
    gb = _native.GBuffer(sc["width"], sc["height"], g.data_ptr(), prim.data_ptr())
    stream = torch.cuda.current_stream().cuda_stream
    for call, (seed, frames) in enumerate([(0, 1), (7, 3)]):
        want = torch.zeros((p, 3), dtype=torch.float32, device="cuda")
        want_res = torch.zeros((p, 4), dtype=torch.int32, device="cuda")
        rl.shade(ctx, scene, g, sc["width"], sc["height"], s, noise_seed=seed, frames=frames, out_rgb=want,
                 reservoirs=want_res, primitive=prim)
        ctx.check()
        got = torch.full((p, 3), -1.0, dtype=torch.float32, device="cuda")
        got_res = torch.zeros((p, 4), dtype=torch.int32, device="cuda")
        nt = _native.NoiseTable(seed)
        st = lib.risltc_shade_noalloc(scene.handle, ctypes.byref(gb), ctypes.byref(s), ctypes.byref(nt), 1, frames,
                                      ctypes.c_void_p(got.data_ptr()), None, ctypes.c_void_p(got_res.data_ptr()),
                                      ctypes.c_void_p(stream))
        assert st == 0, "call %d returned %d" % (call, st)
        assert nt.random_seed == seed + frames
        torch.cuda.synchronize()
        # Exact numerics on both paths: identical bits (the tolerance of the
        # parity tests for exact numerics).
        assert torch.equal(got, want), "call %d" % call
        assert torch.equal(got_res, want_res), "call %d" % call
        if frames == 1:
            # The same frame from the oracle (the reference's routines in C99).
            import oracle
            tris = oracle.triangles_v0e1e2(sc["triangles"])
            osc = oracle.OracleScene(sc["lights"], sc["max_vertex_count"], l0, l1, k, tris)
            orgb, _, _ = oracle.render(osc, oracle.make_settings(candidates=c["candidates"]), sc["gbuffer"],
                                       sc["width"], sc["height"], rl.noise_constants(seed)[0],
                                       primitive=sc["primitive"])
            assert np.array_equal(got.cpu().numpy(), orgb), "call %d against the oracle" % call
    # Frames beyond the static scratch are rejected before any launch.
    big = _native.GBuffer(1024, 512, g.data_ptr(), None)
    nt = _native.NoiseTable(0)
    assert MAX_PIXEL_FRAMES < 1024 * 512
    assert lib.risltc_shade_noalloc(scene.handle, ctypes.byref(big), ctypes.byref(s), ctypes.byref(nt), 1, 1,
                                    ctypes.c_void_p(got.data_ptr()), None, None, ctypes.c_void_p(stream)) == TOO_LARGE
    assert nt.random_seed == 0
    # A scene whose buffers live on another device is rejected before any
    # launch.  With one GPU the other device is faked: the scene's context
    # records its device ordinal first, and the scene points to its context
    # first (static_asserts in api.cu keep that layout).
    ordinal = ctypes.cast(ctypes.cast(scene.handle, ctypes.POINTER(ctypes.c_void_p))[0], ctypes.POINTER(ctypes.c_int))
    assert ordinal[0] == 0
    ordinal[0] = 1
    try:
        st = lib.risltc_shade_noalloc(scene.handle, ctypes.byref(gb), ctypes.byref(s), ctypes.byref(nt), 1, 1,
                                      ctypes.c_void_p(got.data_ptr()), None, None, ctypes.c_void_p(stream))
    finally:
        ordinal[0] = 0
    assert st == INVALID_ARGUMENT and nt.random_seed == 0
    scene.close()
    ctx.close()
