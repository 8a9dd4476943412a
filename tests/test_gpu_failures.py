"""Failure handling without faulting the GPU: every bad input and every
injected allocation failure comes back as a status code and a message, and
the context keeps working afterwards."""
import ctypes as C

import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu


def _expect(ctx, rc, code, text=None):
    assert rc == code, (rc, ctx.lib.gb_last_error(ctx.h))
    if text:
        assert text in ctx.lib.gb_last_error(ctx.h).decode()


def _create(ctx, sc):
    desc, keep = gbpt.make_scene_desc(sc)
    h = C.c_void_p()
    rc = ctx.lib.gb_scene_create(ctx.h, C.byref(desc), C.byref(h))
    return rc, h, keep


def test_bad_scenes_are_rejected(gpu_ctx):
    sc = scenes.cornell(width=16, height=16, spp=1, max_bounces=2)
    bad = scenes.cornell()
    bad.positions = bad.positions.copy()
    bad.positions[3, 4] = np.nan
    rc, _, _ = _create(gpu_ctx, bad)
    _expect(gpu_ctx, rc, gbpt.GB_ERR_INVALID, "non-finite")
    bad = scenes.cornell()
    bad.material_index = bad.material_index.copy()
    bad.material_index[0] = 99
    rc, _, _ = _create(gpu_ctx, bad)
    _expect(gpu_ctx, rc, gbpt.GB_ERR_INVALID, "material index")
    bad = scenes.cornell()
    bad.lights = [dict(bad.lights[0], type=gbpt.GB_LIGHT_SKY)]  # a sky light without a map
    rc, _, _ = _create(gpu_ctx, bad)
    _expect(gpu_ctx, rc, gbpt.GB_ERR_INVALID, "valid map")
    bad.lights = [dict(bad.lights[0], type=7)]
    rc, _, _ = _create(gpu_ctx, bad)
    _expect(gpu_ctx, rc, gbpt.GB_ERR_UNSUPPORTED, "light type")
    # the context still renders
    scene = gpu_ctx.scene(sc)
    img = scene.render(sc.camera, sc.render)
    assert np.isfinite(img).all()
    scene.close()


def test_bad_render_requests_are_rejected(gpu_ctx):
    sc = scenes.cornell(width=16, height=16, spp=1, max_bounces=2)
    scene = gpu_ctx.scene(sc)
    lib = gpu_ctx.lib
    out = np.zeros(16 * 16 * 3, np.float32)
    for change, text in [({"width": 0}, "resolution"), ({"width": 1 << 15, "height": 1 << 15}, "resolution"),
                         ({"spp": 0}, "spp"), ({"max_bounces": 5000}, "spp"), ({"rng_mode": 7}, "rng_mode")]:
        rd = gbpt.make_render_desc(dict(sc.render, **change))
        rc = lib.gb_render(gpu_ctx.h, scene.h, C.byref(gbpt.make_camera(sc.camera)), C.byref(rd),
                           out.ctypes.data_as(C.c_void_p), 0)
        _expect(gpu_ctx, rc, gbpt.GB_ERR_INVALID, text)
    cam = gbpt.make_camera(dict(sc.camera, fovy_deg=0.0))
    rc = lib.gb_render(gpu_ctx.h, scene.h, C.byref(cam), C.byref(gbpt.make_render_desc(sc.render)),
                       out.ctypes.data_as(C.c_void_p), 0)
    _expect(gpu_ctx, rc, gbpt.GB_ERR_INVALID, "fovy")
    rc = lib.gb_render_step(gpu_ctx.h, -1)
    assert rc == gbpt.GB_ERR_INVALID
    scene.close()


def test_injected_allocation_failures():
    """Each of the first allocations of a fresh render fails once in turn;
    the call reports GB_ERR_OOM and the same context then renders the frame
    correctly."""
    ctx = gbpt.Context(0)
    try:
        sc = scenes.cornell(width=24, height=24, spp=2, max_bounces=3)
        scene = ctx.scene(sc)
        good = scene.render(sc.camera, sc.render)
        lib = ctx.lib
        for k in range(0, 12, 3):
            ctx2 = gbpt.Context(0)
            scene2 = ctx2.scene(sc)
            lib.gb_set_fault_injection(k)
            out = np.zeros_like(good)
            rc = lib.gb_render(ctx2.h, scene2.h, C.byref(gbpt.make_camera(sc.camera)),
                               C.byref(gbpt.make_render_desc(sc.render)), out.ctypes.data_as(C.c_void_p), 0)
            lib.gb_set_fault_injection(-1)
            assert rc == gbpt.GB_ERR_OOM, (k, rc)
            assert np.array_equal(scene2.render(sc.camera, sc.render), good)
            scene2.close()
            ctx2.close()
        lib.gb_set_fault_injection(0)
        rc, h, keep = _create(ctx, sc)
        lib.gb_set_fault_injection(-1)
        assert rc == gbpt.GB_ERR_OOM
        scene.close()
    finally:
        gbpt.load_library().gb_set_fault_injection(-1)
        ctx.close()


def test_bad_fitting_and_tuning_requests_are_rejected():
    """gb_ctx_set_gradient_terms, gb_ctx_set_tuning (stack depth, block
    shape), gb_fit_prepare and gb_fit_step refuse bad arguments with
    GB_ERR_INVALID and a message, and the context keeps working."""
    import torch
    ctx = gbpt.Context(0)
    lib = ctx.lib
    try:
        _expect(ctx, lib.gb_ctx_set_gradient_terms(ctx.h, 2), gbpt.GB_ERR_INVALID, "sampling")
        for field, val in (("stack_depth", 16), ("block_threads", 96)):
            t = gbpt.Tuning()
            setattr(t, field, val)
            _expect(ctx, lib.gb_ctx_set_tuning(ctx.h, C.byref(t)), gbpt.GB_ERR_INVALID, field)
        # a step before any gb_fit_prepare
        p = (C.c_void_p * 1)()
        g = (C.c_void_p * 1)()
        _expect(ctx, lib.gb_fit_step(ctx.h, p, g, None), gbpt.GB_ERR_INVALID, "no fitting step prepared")
        sc = scenes.cornell(width=16, height=16, spp=1, max_bounces=2)
        sc.render["rng_mode"] = gbpt.GB_RNG_MRG32K3A_POOL
        h = ctx.scene(sc)
        target = torch.zeros((16, 16, 3), device="cuda")
        _expect(ctx, lib.gb_fit_prepare(ctx.h, 0, None), gbpt.GB_ERR_INVALID, "1..1024")
        with pytest.raises(gbpt.GBError):
            ctx.fit_prepare([(h, sc.camera, sc.render)] * 2, [target.data_ptr()] * 2)
        assert "twice" in lib.gb_last_error(ctx.h).decode()
        ctx.fit_prepare([(h, sc.camera, sc.render)], [target.data_ptr()])
        x = h.get_params()
        bad = x.copy()
        bad[0] = np.nan
        with pytest.raises(gbpt.GBError):
            ctx.fit_step([bad])
        assert "non-finite" in lib.gb_last_error(ctx.h).decode()
        grads, loss = ctx.fit_step([x])
        assert np.isfinite(grads[0]).all() and np.isfinite(loss).all()
        h.close()
    finally:
        ctx.close()
