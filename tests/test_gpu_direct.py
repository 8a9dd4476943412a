"""Direct lighting (gb_render_direct, the reference's gpu_area_lights) against
the oracle's restatement, fed the same MRG32k3a pools: rect lights, a sky
light (uniform-hemisphere sky samples and the sky seen by missed pixels),
and the sample-count edge cases."""
import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu


def _pair(ctx, sc, cam, rd, samples):
    from oracle import oracle
    s = ctx.scene(sc)
    img = s.render_direct(cam, rd, samples)
    s.close()
    n = rd["width"] * rd["height"]
    pool = ctx.mrg_pool(n, max(1, samples - 1), seed=rd.get("seed", 0))
    ref = oracle.OracleScene(sc, use_bvh=True).render_direct(cam, rd, samples, pool)
    return img, ref


@pytest.mark.parametrize("samples", [1, 2, 7])
def test_direct_cornell(gpu_ctx, samples):
    sc = scenes.cornell(width=48, height=40)
    rd = dict(sc.render, shadow_offset=1e-3)
    img, ref = _pair(gpu_ctx, sc, sc.camera, rd, samples)
    assert np.array_equal(img, ref)
    assert img.mean() > 1e-3


def test_direct_icospheres_with_sky(gpu_ctx):
    sc = scenes.icospheres(n_spheres=30, level=2, box=12.0, width=40, height=32, n_lights=2)
    sc.lights.append({"type": gbpt.GB_LIGHT_SKY, "map": scenes.procedural_sky(32, 16), "scale": 0.2,
                      "diameter": 40.0, "power": -1.0})
    rd = dict(sc.render, shadow_offset=0.01, seed=3)
    img, ref = _pair(gpu_ctx, sc, sc.camera, rd, 5)
    assert np.array_equal(img, ref)


def test_direct_rejects_bad_sample_count(gpu_ctx):
    sc = scenes.cornell(width=8, height=8)
    s = gpu_ctx.scene(sc)
    with pytest.raises(gbpt.GBError):
        s.render_direct(sc.camera, sc.render, 0)
    s.close()


def _hybrid_pair(ctx, sc, cam, rd, cs, ls):
    from oracle import oracle
    s = ctx.scene(sc)
    img = s.render_hybrid_direct(cam, rd, cs, ls)
    s.close()
    n = rd["width"] * rd["height"]
    pool = ctx.mrg_pool(n, max(cs, cs * ls), seed=rd.get("seed", 0))
    ref = oracle.OracleScene(sc, use_bvh=True).render_hybrid_direct(cam, rd, cs, ls, pool)
    return img, ref


@pytest.mark.parametrize("cs,ls", [(1, 1), (2, 3), (3, 2)])
def test_hybrid_direct_cornell(gpu_ctx, cs, ls):
    """hybrid_area_lights: jittered camera samples x CPU-sampler light samples."""
    sc = scenes.cornell(width=40, height=32)
    rd = dict(sc.render, seed=1)
    img, ref = _hybrid_pair(gpu_ctx, sc, sc.camera, rd, cs, ls)
    assert np.array_equal(img, ref)
    assert img.mean() > 1e-3


def test_hybrid_direct_lens_sky_and_textures(gpu_ctx):
    sc = scenes.with_textures(scenes.icospheres(n_spheres=30, level=2, box=12.0, width=40, height=32, n_lights=2),
                              fraction=0.5, scale=0.5)
    sc.lights.append({"type": gbpt.GB_LIGHT_SKY, "map": scenes.procedural_sky(32, 16), "scale": 0.2,
                      "diameter": 40.0, "power": -1.0})
    cam = dict(sc.camera, aperture=0.05, focus_distance=30.0)
    rd = dict(sc.render, shadow_offset=0.01, seed=3)
    img, ref = _hybrid_pair(gpu_ctx, sc, cam, rd, 2, 3)
    assert np.array_equal(img, ref)
