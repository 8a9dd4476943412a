"""gb_render_noalloc: the frame of gb_render for callers that must not
allocate device memory while they render (for example a render loop that
shares the GPU with work whose memory lives in its own pool, where a
cudaMalloc/cudaFree would synchronise the device).  Its wavefront state sits
in one fixed device array of the library instead of context buffers.

Checked through the C ABI against gb_render on two calls in a row (the
array keeps the previous call's contents, which must not leak into the
next frame), plus the size limit.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-4
ATOL = 1e-6


def _close(a, b):
    diff = np.abs(a.astype(np.float64) - b)
    assert not (diff > RTOL * np.abs(b) + ATOL).any(), f"max abs diff {diff.max():.3g}"


def test_noalloc_matches_gb_render_twice():
    import torch
    ctx = gbpt.Context(0)
    try:
        lib = ctx.lib
        cases = [scenes.cornell(width=64, height=48, spp=4, max_bounces=5),
                 scenes.icospheres(n_spheres=30, level=3, box=15.0, width=48, height=40, spp=3, max_bounces=6)]
        for sc in cases:
            scene = ctx.scene(sc)
            ref = scene.render(sc.camera, sc.render)
            cam, desc = gbpt.make_camera(sc.camera), gbpt.make_render_desc(sc.render)
            stream = torch.cuda.current_stream()
            for _ in range(2):
                out = torch.full((desc.height, desc.width, 3), float("nan"), device="cuda", dtype=torch.float32)
                rc = lib.gb_render_noalloc(scene.h, C.byref(cam), C.byref(desc), C.c_void_p(out.data_ptr()),
                                           C.c_void_p(stream.cuda_stream))
                assert rc == gbpt.GB_OK, lib.gb_last_error(ctx.h).decode()
                torch.cuda.synchronize()
                _close(out.cpu().numpy(), ref)
            scene.close()
    finally:
        ctx.close()


def test_noalloc_rejects_frames_above_the_limit():
    ctx = gbpt.Context(0)
    try:
        sc = scenes.cornell(width=257, height=256, spp=1, max_bounces=2)
        scene = ctx.scene(sc)
        cam, desc = gbpt.make_camera(sc.camera), gbpt.make_render_desc(sc.render)
        rc = ctx.lib.gb_render_noalloc(scene.h, C.byref(cam), C.byref(desc), C.c_void_p(16), None)
        assert rc == gbpt.GB_ERR_INVALID
        assert b"65536" in ctx.lib.gb_last_error(ctx.h)
        scene.close()
    finally:
        ctx.close()
