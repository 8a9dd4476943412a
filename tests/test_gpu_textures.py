"""Diffuse textures with ray-differential mip selection (material.h:88-170,
hybrid-pt.cpp:300-328, material-cpu.cpp:36-77): GPU frames against the
oracle's restatement, fed the same MRG32k3a pools, bit for bit; textured and
plain scenes in one batch; direct lighting with textures; and the calls that
do not cover textures refusing them."""
import ctypes as C

import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu


def _pair(ctx, sc, rd):
    from oracle import oracle
    s = ctx.scene(sc)
    img = s.render(sc.camera, rd)
    s.close()
    n = rd["width"] * rd["height"]
    pool = ctx.mrg_pool(n, rd["spp"] * rd["max_bounces"], seed=rd.get("seed", 0))
    ref = oracle.OracleScene(sc, use_bvh=False).render(sc.camera, rd, pool)
    return img, ref


@pytest.mark.parametrize("rng_mode", [gbpt.GB_RNG_HALTON_LIGHT, gbpt.GB_RNG_MRG32K3A_POOL])
def test_textured_cornell_frame(gpu_ctx, rng_mode):
    sc = scenes.with_textures(scenes.cornell(width=64, height=48, spp=4, max_bounces=5), fraction=0.7, scale=2.0)
    rd = dict(sc.render, rng_mode=rng_mode)
    img, ref = _pair(gpu_ctx, sc, rd)
    assert np.array_equal(img, ref.astype(np.float32)), np.abs(img - ref).max()
    plain, _ = _pair(gpu_ctx, scenes.cornell(width=64, height=48, spp=4, max_bounces=5), rd)
    assert not np.array_equal(img, plain)


def test_textured_principled_icospheres_frame(gpu_ctx):
    base = scenes.icospheres(n_spheres=20, level=2, box=10.0, width=48, height=32, spp=3, max_bounces=4, n_lights=2)
    sc = scenes.with_textures(base, n_textures=3, size=32, fraction=0.6, scale=0.5, seed=5)
    assert any(m["principled"] >= 0 and m["diffuse_texture"] >= 0 for m in sc.materials)
    img, ref = _pair(gpu_ctx, sc, dict(sc.render))
    assert np.array_equal(img, ref.astype(np.float32)), np.abs(img - ref).max()


def test_textured_and_plain_scenes_in_one_batch(gpu_ctx):
    a = scenes.with_textures(scenes.cornell(width=40, height=32, spp=3, max_bounces=4), fraction=1.0, scale=3.0)
    b = scenes.cornell(width=24, height=24, spp=2, max_bounces=3, seed=2)
    sa, sb = gpu_ctx.scene(a), gpu_ctx.scene(b)
    single = [sa.render(a.camera, a.render), sb.render(b.camera, b.render)]
    for graph in (False, True):
        out = gpu_ctx.render_batch([(sa, a.camera, a.render), (sb, b.camera, b.render)], graph=graph)
        assert all(np.array_equal(x, y) for x, y in zip(out, single))
    sa.close()
    sb.close()


def test_textured_direct_lighting(gpu_ctx):
    from oracle import oracle
    sc = scenes.with_textures(scenes.cornell(width=48, height=40), fraction=1.0, scale=2.0)
    rd = dict(sc.render, shadow_offset=1e-3)
    s = gpu_ctx.scene(sc)
    img = s.render_direct(sc.camera, rd, 4)
    s.close()
    pool = gpu_ctx.mrg_pool(48 * 40, 3, seed=0)
    ref = oracle.OracleScene(sc, use_bvh=True).render_direct(sc.camera, rd, 4, pool)
    assert np.array_equal(img, ref)


def test_texture_errors(gpu_ctx):
    sc = scenes.with_textures(scenes.cornell(width=16, height=16, spp=1, max_bounces=2), fraction=1.0)
    bad = scenes.SceneData(**{**sc.__dict__, "materials": [dict(m, diffuse_texture=5) for m in sc.materials]})
    with pytest.raises(gbpt.GBError, match="texture index"):
        gpu_ctx.scene(bad)
    with pytest.raises(gbpt.GBError, match="texture coordinates"):
        gpu_ctx.scene(scenes.SceneData(**{**sc.__dict__, "texcoords": None}))
    tc = sc.texcoords.copy()
    tc[3, 1] = np.nan
    with pytest.raises(gbpt.GBError, match="non-finite texture"):
        gpu_ctx.scene(scenes.SceneData(**{**sc.__dict__, "texcoords": tc}))
    s = gpu_ctx.scene(sc)
    with pytest.raises(gbpt.GBError) as ei:
        s.backward(sc.camera, sc.render, np.ones((16, 16, 3), np.float32))
    assert ei.value.code == gbpt.GB_ERR_UNSUPPORTED
    cam, desc = gbpt.make_camera(sc.camera), gbpt.make_render_desc(sc.render)
    rc = gpu_ctx.lib.gb_render_noalloc(s.h, C.byref(cam), C.byref(desc), C.c_void_p(16), None)
    assert rc == gbpt.GB_ERR_UNSUPPORTED
    s.close()
