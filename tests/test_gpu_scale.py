"""Parity at the sizes the benchmark runs: the 1,024,010-triangle icosphere
scene (800 displaced icospheres of 1280 triangles + a 10-triangle ground
plane in a 100^3 box, host binned-SAH tree of depth 12), the 256x256 Cornell
room at 16 spp and 5 bounces with Halton light samples, and the largest
member of the 64-scene mixed set rendered inside a batched frame.

Hits must be bit-exact (triangle id, t, beta, gamma) for camera, bounce,
shadow and random rays, with and without finite max_t, through the closest
and any-hit tracers (tracers.cu:38-140 tie rule: the (t, id) minimum).
Frames must agree with the oracle's restatement of the hybrid bouncer
(hybrid-pt.h:115-249, hybrid-pt.cpp:450-584) per pixel within 1e-4
relative (absolute floor 1e-6) on the same MRG32k3a pools."""
import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-4
ATOL = 1e-6
FLT_MAX = np.float32(3.4028235e38)


def _compare(img, ref, what):
    assert img.shape == ref.shape
    assert np.isfinite(img).all()
    diff = np.abs(img.astype(np.float64) - ref)
    bad = diff > RTOL * np.abs(ref) + ATOL
    assert not bad.any(), f"{what}: {bad.any(axis=2).sum()} pixels differ, max abs diff {diff.max():.3g}"


def _fp64_refs():
    from pathlib import Path
    p = Path(__file__).resolve().parent / "golden" / "fp64_refs.npz"
    return dict(np.load(p))


def _against_fp64(img, key, spp):
    """A GPU frame (the fixture's rows) against the converged fp64 image of
    the oracle's independent double-precision restatement: the mean within
    4 standard errors (no bias) and the RMSE the noise of spp + the
    reference's samples predicts (var = one-sample variance)."""
    g = _fp64_refs()
    ref = g[key].astype(np.float64)
    n_ref, var = int(g[key + "_spp"]), float(g[key + "_var"].mean())
    x = img.astype(np.float64)
    assert x.shape == ref.shape
    se = np.sqrt(var * (1.0 / spp + 1.0 / n_ref) / x.size)
    z = (x.mean() - ref.mean()) / se
    rmse = float(np.sqrt(np.mean((x - ref) ** 2)))
    expected = float(np.sqrt(var * (1.0 / spp + 1.0 / n_ref)))
    assert abs(z) < 4.0, f"{key}: GPU mean {x.mean():.5f}, fp64 {ref.mean():.5f}, z = {z:.2f}"
    assert 0.75 < rmse / expected < 1.33, f"{key}: RMSE {rmse:.5f}, noise predicts {expected:.5f}"
    return rmse, expected


def _check_hits(g, o, what):
    assert np.array_equal(g["ref"], o["ref"]), f"{what}: {(g['ref'] != o['ref']).sum()} triangle ids differ"
    hit = o["ref"] != 0xFFFFFFFF
    for k in ("t", "beta", "gamma"):
        assert np.array_equal(g[k][hit].view(np.uint32), o[k][hit].view(np.uint32)), f"{what}: {k}"


@pytest.fixture(scope="module")
def c1(gpu_ctx):
    from oracle import oracle
    sc = scenes.icospheres()
    assert sc.num_triangles == 1_024_010
    scene = gpu_ctx.scene(sc)
    info = scene.info()
    orc = oracle.OracleScene(sc, use_bvh=True)
    yield sc, scene, orc, info
    scene.close()
    orc.close()


def _camera_rays(cam, w, h, n, rng):
    """Pinhole rays through random points of random pixels (the Shirley
    camera of raygen.cu:61-118, evaluated in numpy)."""
    pos = np.array(cam["pos"], np.float64)
    W = np.array(cam["dir"], np.float64)
    W /= np.linalg.norm(W)
    U = np.cross(np.array(cam["up"], np.float64), W)
    U /= np.linalg.norm(U)
    V = np.cross(W, U)
    th = np.tan(np.pi * cam["fovy_deg"] / 2.0 / 180.0)
    tw = th * w / h
    x = rng.uniform(0, w, n)
    y = rng.uniform(0, h, n)
    u = (x / w * 2.0 - 1.0) * tw
    v = (y / h * 2.0 - 1.0) * th
    d = u[:, None] * U + v[:, None] * V + W
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.broadcast_to(pos, d.shape).astype(np.float32), d.astype(np.float32)


def _bounce_rays(sc, o, d, hits, offset, rng):
    """Rays leaving the hit points of (o, d) into the hemisphere on the
    incident side, from an origin moved `offset` along the face normal (the
    reference's next-ray set-up, hybrid-pt.cpp:551-555)."""
    hit = hits["ref"] != 0xFFFFFFFF
    ids = hits["ref"][hit].astype(np.int64)
    p = sc.positions[ids].reshape(-1, 3, 3).astype(np.float64)
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    dd = d[hit].astype(np.float64)
    n *= -np.sign(np.sum(n * dd, axis=1))[:, None]
    P = o[hit] + hits["t"][hit][:, None].astype(np.float64) * dd
    org = P + offset * n
    r = rng.normal(size=org.shape)
    r /= np.linalg.norm(r, axis=1, keepdims=True)
    r *= np.sign(np.sum(r * n, axis=1))[:, None]
    return org.astype(np.float32), r.astype(np.float32)


def _shadow_rays(sc, org, rng):
    """Rays from `org` to random points of random area lights, max_t = the
    distance (arealight-sampler-cpu.cpp:69-119 without the origin offset)."""
    L = sc.lights
    k = rng.integers(0, len(L), org.shape[0])
    c = np.array([L[i]["center"] for i in k], np.float64)
    wh = np.array([L[i]["wh"] for i in k], np.float64)
    s = c + (rng.uniform(-0.5, 0.5, (org.shape[0], 2)) * wh) @ np.array([[1.0, 0, 0], [0, 0, 1.0]])
    v = s - org
    dist = np.linalg.norm(v, axis=1)
    return (v / dist[:, None]).astype(np.float32), dist.astype(np.float32)


def test_c1_tree_shape(c1):
    """The tree the benchmark's roofline is measured on: deep enough for the
    32-entry stack and the per-node exponents to matter."""
    _, _, _, info = c1
    assert info["num_triangles"] == 1_024_010
    assert info["depth"] >= 10 and info["num_nodes"] > 100_000


def test_c1_hits_bit_exact(gpu_ctx, c1):
    """>= 400 K rays of every kind against the 1 M-triangle tree: camera
    rays, bounce rays from their hits, shadow rays to the lights, random
    rays from outside the scene; each set also with finite max_t cut before,
    at and beyond the hit.  Closest hits bit-exact, any-hit equal."""
    sc, scene, orc, _ = c1
    rng = np.random.default_rng(2024)
    W, H = sc.render["width"], sc.render["height"]
    co, cd = _camera_rays(sc.camera, W, H, 120_000, rng)
    tinf = np.full(co.shape[0], FLT_MAX, np.float32)
    g = scene.trace_closest(co, cd, tinf)
    _check_hits(g, orc.trace_closest(co, cd, tinf), "camera rays")
    assert (g["ref"] != 0xFFFFFFFF).mean() > 0.3
    bo, bd = _bounce_rays(sc, co, cd, g, sc.render["ray_offset"], rng)
    so, sd = _bounce_rays(sc, co, cd, g, sc.render["shadow_offset"], rng)
    ld, ldist = _shadow_rays(sc, so, rng)
    ro, rd = scenes.random_rays(sc, 120_000, seed=77)
    sets = [("camera", co, cd, g["t"]), ("bounce", bo, bd, None), ("random", ro, rd, None)]
    total = 0
    for name, o, d, t_hit in sets:
        n = o.shape[0]
        inf = np.full(n, FLT_MAX, np.float32)
        gh = scene.trace_closest(o, d, inf)
        _check_hits(gh, orc.trace_closest(o, d, inf), name)
        # finite max_t: before, at and beyond the hit distance
        th = gh["t"].copy()
        th[gh["ref"] == 0xFFFFFFFF] = 150.0
        f = rng.uniform(0.5, 1.5, n).astype(np.float32)
        tm = (th * f).astype(np.float32)
        tm[::5] = th[::5]  # exactly the hit distance: t <= max_t keeps it
        _check_hits(scene.trace_closest(o, d, tm), orc.trace_closest(o, d, tm), name + " finite max_t")
        assert np.array_equal(scene.trace_any(o, d, tm), orc.trace_any(o, d, tm)), name + " any-hit"
        total += 2 * n
    gs = scene.trace_closest(so, ld, ldist)
    _check_hits(gs, orc.trace_closest(so, ld, ldist), "shadow")
    occ = scene.trace_any(so, ld, ldist)
    assert np.array_equal(occ, orc.trace_any(so, ld, ldist)), "shadow any-hit"
    assert 0.05 < occ.mean() < 0.95
    total += so.shape[0]
    assert total >= 400_000


def test_c1_frame_2spp_full(gpu_ctx, c1):
    """The whole 1280x720 frame of the benchmark (8 bounces, Russian roulette
    from bounce 3) at 2 spp, every pixel against the oracle."""
    from oracle import oracle  # noqa: F401
    sc, scene, orc, _ = c1
    rd = dict(sc.render, spp=2)
    img = scene.render(sc.camera, rd)
    st = gpu_ctx.stats()
    pool = gpu_ctx.mrg_pool(rd["width"] * rd["height"], rd["spp"] * rd["max_bounces"])
    ref, ost = orc.render(sc.camera, rd, pool, with_stats=True)
    _compare(img, ref, "C1 2 spp")
    assert st["camera_rays"] == int(ost[0]) and st["extension_rays"] == int(ost[1])
    assert (img != 1.0).any(axis=2).mean() > 0.3


def test_c1_band_64spp(gpu_ctx, c1):
    """A full-width band of 16 rows through the middle of the benchmark frame
    at its full 64 spp: the exact frame the bench times."""
    sc, scene, orc, _ = c1
    rd = dict(sc.render)
    assert rd["spp"] == 64 and rd["max_bounces"] == 8 and rd["rr_start"] == 3
    img = scene.render(sc.camera, rd)
    W = rd["width"]
    r0, r1 = 352, 368
    pool = gpu_ctx.mrg_pool((r1 - r0) * W, rd["spp"] * rd["max_bounces"], pixel0=r0 * W)
    ref = orc.render(sc.camera, rd, pool, r0, r1)
    _compare(img[r0:r1], ref, "C1 64 spp band")
    g = _fp64_refs()
    assert tuple(g["c1_rows"]) == (r0, r1)
    _against_fp64(img[r0:r1], "c1", rd["spp"])


@pytest.mark.parametrize("rng_mode", [gbpt.GB_RNG_HALTON_LIGHT, gbpt.GB_RNG_MRG32K3A_POOL])
def test_c0_cornell_full_size(gpu_ctx, rng_mode):
    """The CPU-runnable configuration at its stated size: 256x256, 16 spp,
    5 bounces, light samples from the Halton pool (util.cpp:38-51), path
    draws from curand MRG32k3a seeded by pixel (util-kernels.cu:284)."""
    from oracle import oracle
    sc = scenes.cornell()
    rd = dict(sc.render, rng_mode=rng_mode)
    assert (rd["width"], rd["height"], rd["spp"], rd["max_bounces"]) == (256, 256, 16, 5)
    assert sc.num_triangles == 48
    scene = gpu_ctx.scene(sc)
    img = scene.render(sc.camera, rd)
    scene.close()
    pool = gpu_ctx.mrg_pool(256 * 256, rd["spp"] * rd["max_bounces"])
    ref = oracle.OracleScene(sc, use_bvh=False).render(sc.camera, rd, pool)
    _compare(img, ref, "C0")
    assert img.mean() > 0.05
    if rng_mode == gbpt.GB_RNG_HALTON_LIGHT:  # the configuration's light draws
        _against_fp64(img, "c0", rd["spp"])


def test_c2_largest_member_in_batch(gpu_ctx):
    """The largest scene of the 64-scene mixed set (430 K triangles), rendered
    in one batched CUDA-graph frame together with three other members; its
    image against the oracle over a band of rows (full width, all spp)."""
    from oracle import oracle
    mixed = scenes.mixed_set()
    sizes = [s.num_triangles for s in mixed]
    big = int(np.argmax(sizes))
    assert sizes[big] > 400_000
    others = [i for i in np.random.default_rng(1).choice(len(mixed), 6, replace=False) if i != big][:3]
    pick = [big] + [int(i) for i in others]
    handles = [gpu_ctx.scene(mixed[i]) for i in pick]
    jobs = [(h, dict(mixed[i].camera), dict(mixed[i].render)) for h, i in zip(handles, pick)]
    imgs = gpu_ctx.render_batch(jobs, graph=True)
    for h in handles:
        h.close()
    sc = mixed[big]
    rd = dict(sc.render)
    W, H = rd["width"], rd["height"]
    rows = min(H, 32)
    r0 = (H - rows) // 2
    pool = gpu_ctx.mrg_pool(rows * W, rd["spp"] * rd["max_bounces"], seed=rd["seed"], pixel0=r0 * W)
    ref = oracle.OracleScene(sc, use_bvh=True).render(sc.camera, rd, pool, r0, r0 + rows)
    _compare(imgs[0][r0:r0 + rows], ref, f"mixed-set scene {big} ({sizes[big]} triangles)")
    assert tuple(_fp64_refs()["c2_rows"]) == (r0, r0 + rows)
    _against_fp64(imgs[0][r0:r0 + rows], "c2", rd["spp"])


def test_adjoint_configuration_frame_against_fp64(gpu_ctx, c1):
    """The forward frame of the differentiation workload (the 1M-triangle
    scene at 512x512, 16 spp, 4 bounces) against its fp64 reference band."""
    sc, scene, _, _ = c1
    rd = dict(sc.render, width=512, height=512, spp=16, max_bounces=4)
    img = scene.render(sc.camera, rd)
    r0, r1 = (int(v) for v in _fp64_refs()["c3_rows"])
    _against_fp64(img[r0:r1], "c3", rd["spp"])
