"""Frame parity: the GPU wavefront frame vs the CPU oracle's restatement of
the hybrid bouncer, fed with the same MRG32k3a pools (gb_mrg_pool: curand
MRG32k3a, seed 0, subsequence = pixel).  Per-pixel radiance must agree
within 1e-4 relative (absolute floor 1e-6); the arithmetic is shared and
IEEE-exact, so in practice the frames are bit-identical."""
import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-4
ATOL = 1e-6


def _compare(img, ref):
    assert img.shape == ref.shape
    assert np.isfinite(img).all()
    diff = np.abs(img.astype(np.float64) - ref)
    bad = diff > RTOL * np.abs(ref) + ATOL
    assert not bad.any(), f"{bad.any(axis=2).sum()} pixels differ, max abs diff {diff.max():.3g}"


def _render_pair(ctx, sc, rd, use_bvh=True):
    from oracle import oracle
    scene = ctx.scene(sc)
    img = scene.render(sc.camera, rd)
    npx = rd["width"] * rd["height"]
    pool = ctx.mrg_pool(npx, rd["spp"] * rd["max_bounces"], seed=rd.get("seed", 0))
    ref = oracle.OracleScene(sc, use_bvh=use_bvh).render(sc.camera, rd, pool)
    scene.close()
    return img, ref


@pytest.mark.parametrize("rng_mode", [gbpt.GB_RNG_HALTON_LIGHT, gbpt.GB_RNG_MRG32K3A_POOL])
def test_cornell_frame(gpu_ctx, rng_mode):
    sc = scenes.cornell(width=64, height=48, spp=4, max_bounces=5)
    rd = dict(sc.render, rng_mode=rng_mode)
    img, ref = _render_pair(gpu_ctx, sc, rd, use_bvh=False)
    _compare(img, ref)
    assert img.mean() > 0.01


def test_icospheres_frame_principled(gpu_ctx):
    sc = scenes.icospheres(n_spheres=60, level=3, box=20.0, width=80, height=45, spp=3, max_bounces=6,
                           rr_start=-1)
    rd = dict(sc.render)
    img, ref = _render_pair(gpu_ctx, sc, rd)
    _compare(img, ref)


def test_icospheres_frame_russian_roulette(gpu_ctx):
    sc = scenes.icospheres(n_spheres=60, level=3, box=20.0, width=64, height=40, spp=2, max_bounces=8, rr_start=2)
    rd = dict(sc.render)
    img, ref = _render_pair(gpu_ctx, sc, rd)
    _compare(img, ref)


def test_thin_lens_frame(gpu_ctx):
    sc = scenes.cornell(width=40, height=40, spp=3, max_bounces=3)
    cam = dict(sc.camera, aperture=0.05, focus_distance=1.9)
    rd = dict(sc.render, rng_mode=gbpt.GB_RNG_MRG32K3A_POOL)
    from oracle import oracle
    scene = gpu_ctx.scene(sc)
    img = scene.render(cam, rd)
    pool = gpu_ctx.mrg_pool(40 * 40, rd["spp"] * rd["max_bounces"])
    ref = oracle.OracleScene(sc, use_bvh=False).render(cam, rd, pool)
    scene.close()
    _compare(img, ref)


def test_progressive_steps_match_full_frame(gpu_ctx):
    """gb_render_begin/step/read (gi_algorithm::update form) == gb_render."""
    import ctypes as C
    sc = scenes.cornell(width=32, height=32, spp=4, max_bounces=4)
    rd = dict(sc.render)
    scene = gpu_ctx.scene(sc)
    full = scene.render(sc.camera, rd)
    lib = gpu_ctx.lib
    cam, desc = gbpt.make_camera(sc.camera), gbpt.make_render_desc(rd)
    gpu_ctx.check(lib.gb_render_begin(gpu_ctx.h, scene.h, C.byref(cam), C.byref(desc)))
    done = C.c_int()
    for _ in range(4):
        gpu_ctx.check(lib.gb_render_step(gpu_ctx.h, 1))
    gpu_ctx.check(lib.gb_render_paths_done(gpu_ctx.h, C.byref(done)))
    assert done.value == 4
    out = np.empty_like(full)
    gpu_ctx.check(lib.gb_render_read(gpu_ctx.h, out.ctypes.data_as(C.c_void_p), 0))
    assert np.array_equal(out, full)
    scene.close()


def test_determinism_and_stats(gpu_ctx):
    sc = scenes.cornell(width=48, height=48, spp=2, max_bounces=3)
    scene = gpu_ctx.scene(sc)
    a = scene.render(sc.camera, sc.render)
    s1 = gpu_ctx.stats()
    b = scene.render(sc.camera, sc.render, instrumented=True)
    s2 = gpu_ctx.stats()
    scene.close()
    assert np.array_equal(a, b)
    assert s1["camera_rays"] == 48 * 48 * 2
    assert s1["extension_rays"] == s2["extension_rays"] and s1["shadow_rays"] == s2["shadow_rays"]
    assert s2["closest_node_visits"] > 0 and s2["closest_tri_tests"] > 0 and s2["shadow_node_visits"] > 0


def test_mrg_pool_streams(gpu_ctx):
    """Update u of pixel i = draws 3u..3u+2 of curand MRG32k3a(seed, i): a later
    window equals the tail of a longer one, values lie in (0, 1]."""
    a = gpu_ctx.mrg_pool(100, 6)
    b = gpu_ctx.mrg_pool(100, 2, first_update=4)
    assert np.array_equal(a[4:], b)
    assert (a > 0).all() and (a <= 1).all()
    assert not np.array_equal(a[0, 0], a[0, 1])


def test_mrg_stream_jump_matches_curand_init(gpu_ctx):
    """The library's stream starts (subsequence i = i * 2^76 steps, by jump
    matrices) equal curand_init(seed, i, 0): small indices, every single bit,
    every all-ones prefix and random 32-bit indices, for several seeds."""
    rng = np.random.default_rng(5)
    sub = np.concatenate([np.arange(4096, dtype=np.uint64), np.uint64(1) << np.arange(32, dtype=np.uint64),
                          (np.uint64(1) << np.arange(1, 33, dtype=np.uint64)) - np.uint64(1),
                          rng.integers(0, 2**32, 20000, dtype=np.uint64)]).astype(np.uint32)
    for seed in (0, 1, 0x9E3779B9):
        a = gpu_ctx.mrg_states(sub, seed=seed, method=0)
        b = gpu_ctx.mrg_states(sub, seed=seed, method=1)
        assert np.array_equal(a, b), seed
    assert not np.array_equal(a[0], a[1])


def test_ingested_obj_scene_frame(gpu_ctx):
    """A scene gathered by gb_asset (OBJ + MTL + .pbrdf + light script),
    created straight from gb_asset_get_desc's description, renders the
    oracle's frame."""
    import ctypes as C
    from pathlib import Path
    assets = Path(__file__).resolve().parent / "golden" / "assets"
    a = gbpt.Asset()
    a.add_obj(assets / "room.obj", assets / "materials")
    a.add_lights(assets / "room.lights.scm")
    cam = {"pos": (2.0, 1.5, -3.0), "dir": (0.0, -0.1, 1.0), "up": (0.0, 1.0, 0.0), "fovy_deg": 50.0}
    rd = {"width": 48, "height": 40, "spp": 3, "max_bounces": 4, "rng_mode": gbpt.GB_RNG_MRG32K3A_POOL, "seed": 0,
          "ray_offset": 1e-3, "shadow_offset": 1e-3, "rr_start": -1}
    desc = gbpt.SceneDesc()
    assert gpu_ctx.lib.gb_asset_get_desc(a.h, C.byref(desc)) == gbpt.GB_OK
    h = C.c_void_p()
    gpu_ctx.check(gpu_ctx.lib.gb_scene_create(gpu_ctx.h, C.byref(desc), C.byref(h)))
    img = np.empty((40, 48, 3), np.float32)
    gpu_ctx.check(gpu_ctx.lib.gb_render(gpu_ctx.h, h, C.byref(gbpt.make_camera(cam)), C.byref(gbpt.make_render_desc(rd)),
                                        img.ctypes.data_as(C.c_void_p), 0))
    gpu_ctx.lib.gb_scene_destroy(h)
    sd = a.scene_data(cam, rd)
    a.close()
    from oracle import oracle
    pool = gpu_ctx.mrg_pool(48 * 40, rd["spp"] * rd["max_bounces"])
    ref = oracle.OracleScene(sd, use_bvh=False).render(cam, rd, pool)
    _compare(img, ref)
    assert img.mean() > 1e-3


def test_sky_light_frame(gpu_ctx):
    """A rect light plus a sky light: sky NEE samples (importance-sampled
    lat-long map) and sky lookups of secondary misses, against the oracle."""
    sc = scenes.icospheres(n_spheres=20, level=2, box=12.0, width=48, height=32, spp=3, max_bounces=4, n_lights=1,
                           rr_start=-1)
    sc.lights.append({"type": gbpt.GB_LIGHT_SKY, "map": scenes.procedural_sky(64, 32), "scale": 0.5,
                      "diameter": 30.0, "power": -1.0})
    for mode in (gbpt.GB_RNG_MRG32K3A_POOL, gbpt.GB_RNG_HALTON_LIGHT):
        rd = dict(sc.render, rng_mode=mode)
        img, ref = _render_pair(gpu_ctx, sc, rd)
        _compare(img, ref)
        assert img.mean() > 1e-3


def test_sky_light_errors(gpu_ctx):
    sc = scenes.icospheres(n_spheres=4, level=1, box=6.0, width=16, height=16, spp=1, max_bounces=2, n_lights=1)
    sky = {"type": gbpt.GB_LIGHT_SKY, "map": scenes.procedural_sky(16, 8), "scale": 1.0, "diameter": 10.0,
           "power": -1.0}
    two = scenes.SceneData(sc.positions, sc.normals, sc.material_index, sc.materials, sc.params,
                           sc.lights + [sky, dict(sky)], sc.camera, sc.render)
    with pytest.raises(gbpt.GBError, match="one sky"):
        gpu_ctx.scene(two)
    bad = dict(sky, map=np.full((8, 16, 3), np.nan, np.float32))
    nan = scenes.SceneData(sc.positions, sc.normals, sc.material_index, sc.materials, sc.params,
                           sc.lights + [bad], sc.camera, sc.render)
    with pytest.raises(gbpt.GBError, match="finite"):
        gpu_ctx.scene(nan)
    ok = scenes.SceneData(sc.positions, sc.normals, sc.material_index, sc.materials, sc.params,
                          sc.lights + [sky], sc.camera, sc.render)
    s = gpu_ctx.scene(ok)
    with pytest.raises(gbpt.GBError, match="rectangular"):
        s.backward(sc.camera, sc.render, np.zeros((16, 16, 3), np.float32))
    s.close()


def test_triangle_policies_agree(gpu_ctx):
    """All traversal triangle policies (incl. the warp-cooperative one)
    produce bit-identical frames: the closest hit is the (t, id) minimum
    whatever the visiting order, and any-hit only asks whether one exists."""
    sc = scenes.icospheres(n_spheres=60, level=3, box=20.0, width=64, height=40, spp=3, max_bounces=5, rr_start=2)
    s = gpu_ctx.scene(sc)
    old = gpu_ctx.get_tuning()
    imgs = []
    try:
        for mode in (1, 2, 3, 4):
            gpu_ctx.set_tuning(tri_mode=mode)
            imgs.append(s.render(sc.camera, sc.render))
            st = gpu_ctx.stats()
            assert st["camera_rays"] == 64 * 40 * 3
    finally:
        gpu_ctx.set_tuning(tri_mode=old["tri_mode"])
    for im in imgs[1:]:
        assert np.array_equal(imgs[0], im)
    s.close()


def test_traversal_stack_and_block_variants_agree(gpu_ctx):
    """The traversal kernels built for 24 or 32 stack entries and 64- or
    128-thread blocks (gb_tuning stack_depth / block_threads) render the same
    frame bit for bit, here on a tree of depth 10+ (a stack of 24 entries
    suffices for it; a shallower tree never needs more than its depth
    plus the postponed triangle groups)."""
    sc = scenes.icospheres(n_spheres=300, level=3, box=50.0, width=96, height=54, spp=3, max_bounces=6, rr_start=3)
    s = gpu_ctx.scene(sc)
    old = gpu_ctx.get_tuning()
    imgs = []
    try:
        for stack, block in ((32, 128), (24, 128), (32, 64), (24, 64)):
            gpu_ctx.set_tuning(stack_depth=stack, block_threads=block)
            t = gpu_ctx.get_tuning()
            assert (t["stack_depth"], t["block_threads"]) == (stack, block)
            imgs.append(s.render(sc.camera, sc.render))
    finally:
        gpu_ctx.set_tuning(stack_depth=old["stack_depth"], block_threads=old["block_threads"])
    for im in imgs[1:]:
        assert np.array_equal(imgs[0], im)
    with pytest.raises(gbpt.GBError, match="stack_depth"):
        gpu_ctx.set_tuning(stack_depth=16)
    s.close()
