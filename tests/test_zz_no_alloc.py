"""gb_render_noalloc: the frame of gb_render for callers that must not
allocate device memory while they render.  Such callers are, for example, a
render loop that shares the GPU with work whose memory lives in its own pool
(a cudaMalloc or cudaFree there would synchronise the whole device and
fragment that pool), or a host thread that must not block inside the
driver's allocator.  The entry point keeps its wavefront state in one fixed
device array of the library instead of context buffers.

Checked through the C ABI against gb_render on two calls in a row (the array
keeps the previous call's contents, which must not leak into the next
frame): the images must be bit-identical, no library allocation may happen
(the library's allocation hook is armed to fail the next one), and the
device's free memory must not move across the second call.  Also: the size
limit, the caller's current device after the call, and the refusal to run
while its stream is capturing.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu


def _cases():
    return [
        (scenes.cornell(width=64, height=48, spp=4, max_bounces=5), gbpt.GB_RNG_MRG32K3A_POOL),
        (scenes.cornell(width=64, height=48, spp=4, max_bounces=5), gbpt.GB_RNG_HALTON_LIGHT),
        (scenes.icospheres(n_spheres=30, level=3, box=15.0, width=48, height=40, spp=3, max_bounces=6),
         gbpt.GB_RNG_MRG32K3A_POOL),
    ]


def test_noalloc_matches_gb_render_twice():
    import torch
    ctx = gbpt.Context(0)
    lib = ctx.lib
    try:
        for sc, mode in _cases():
            rd = dict(sc.render, rng_mode=mode)
            scene = ctx.scene(sc)
            ref = scene.render(sc.camera, rd)
            cam, desc = gbpt.make_camera(sc.camera), gbpt.make_render_desc(rd)
            stream = torch.cuda.current_stream()
            out = torch.empty((desc.height, desc.width, 3), device="cuda", dtype=torch.float32)
            torch.cuda.synchronize()
            for call in range(2):
                out.fill_(float("nan"))
                torch.cuda.synchronize()
                free_before = torch.cuda.mem_get_info()[0]
                # any device allocation the library makes from here on fails
                lib.gb_set_fault_injection(0)
                try:
                    rc = lib.gb_render_noalloc(scene.h, C.byref(cam), C.byref(desc), C.c_void_p(out.data_ptr()),
                                               C.c_void_p(stream.cuda_stream))
                finally:
                    lib.gb_set_fault_injection(-1)
                assert rc == gbpt.GB_OK, lib.gb_last_error(ctx.h).decode()
                torch.cuda.synchronize()
                if call == 1:
                    assert torch.cuda.mem_get_info()[0] == free_before
                got = out.cpu().numpy()
                assert np.array_equal(got, ref), f"call {call}: max abs diff {np.nanmax(np.abs(got - ref)):.3g}"
            scene.close()
    finally:
        ctx.close()


@pytest.mark.filterwarnings("ignore:The CUDA Graph is empty")
def test_noalloc_keeps_the_callers_device_and_refuses_capture():
    import torch
    ctx = gbpt.Context(0)
    lib = ctx.lib
    try:
        sc = scenes.cornell(width=16, height=16, spp=1, max_bounces=2)
        scene = ctx.scene(sc)
        cam, desc = gbpt.make_camera(sc.camera), gbpt.make_render_desc(sc.render)
        out = torch.empty((16, 16, 3), device="cuda", dtype=torch.float32)
        torch.cuda.set_device(0)
        stream = torch.cuda.Stream()
        torch.cuda.synchronize()
        assert lib.gb_render_noalloc(scene.h, C.byref(cam), C.byref(desc), C.c_void_p(out.data_ptr()),
                                     C.c_void_p(stream.cuda_stream)) == gbpt.GB_OK
        assert torch.cuda.current_device() == 0
        g = torch.cuda.CUDAGraph()
        rc = None
        with torch.cuda.graph(g, stream=stream):
            rc = lib.gb_render_noalloc(scene.h, C.byref(cam), C.byref(desc), C.c_void_p(out.data_ptr()),
                                       C.c_void_p(stream.cuda_stream))
        assert rc == gbpt.GB_ERR_INVALID
        assert b"capturing" in lib.gb_last_error(ctx.h)
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
