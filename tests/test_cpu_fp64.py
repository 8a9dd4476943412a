"""The oracle's independent double-precision restatement of the hybrid path
(oracle/fp64_render.cpp), which renders the converged reference images the
GPU frames' RMSE is stated against.

It shares no code with the kernels or with the float oracle (own tree, own
random numbers, every formula re-derived from hybrid-pt.cpp,
arealight-sampler-cpu.cpp and principledMaterial.h in double), so agreement
in expectation between it and the float path is an independent check of the
float path's per-path arithmetic: at equal sample counts and different
random numbers, the image means must differ by no more than their noise
(|difference| / standard error < 4), for Lambert and for every principled
lobe (metal, anisotropic metal, sheen, subsurface, clearcoat, glass), with
and without Russian roulette, with MRG32k3a-style and Halton light draws.
The float path is the oracle fed with seeded uniform pools; the GPU frames
equal it bit for bit (tests/test_gpu_*.py).
"""
from pathlib import Path

import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

GOLDEN = Path(__file__).resolve().parent / "golden" / "fp64_refs.npz"


def _pool(spp, L, npx, seed):
    rng = np.random.default_rng(seed)
    return np.maximum(rng.uniform(0.0, 1.0, (spp * L, npx, 3)).astype(np.float32), np.float32(1e-7))


def _mean_z(a, b, var, n_a, n_b):
    """(mean(a) - mean(b)) / its standard error, var = per-pixel one-sample
    variance of the shared estimator."""
    se = np.sqrt(var.sum() * (1.0 / n_a + 1.0 / n_b)) / var.size
    return (a.mean() - b.mean()) / se


def test_fp64_traversal_agrees_with_float_tracer():
    """Same triangle for every ray except exact-distance ties, where the
    (t, id) rule picks the same lower id; t within float rounding."""
    from oracle import oracle
    for sc in (scenes.cornell(), scenes.icospheres(n_spheres=40, level=3, box=20.0)):
        o32 = oracle.OracleScene(sc, use_bvh=True)
        f64 = oracle.F64Scene(sc)
        o, d = scenes.random_rays(sc, 30000, seed=9)
        tmax = np.full(o.shape[0], 3.4e38, np.float32)
        h = o32.trace_closest(o, d, tmax)
        ids, t = f64.trace_closest(o, d, tmax)
        r32 = h["ref"].astype(np.int64)
        r32[r32 == 0xFFFFFFFF] = -1
        assert (r32 == ids).mean() > 0.99
        assert np.array_equal(r32 >= 0, ids >= 0)  # the same rays hit something
        both = (r32 == ids) & (ids >= 0)
        assert np.all(np.abs(h["t"][both] - t[both]) <= 1e-5 * t[both] + 1e-6)
        # rays whose ids differ hit coplanar faces (the room's floor seen from
        # below, where the boxes' bottoms lie in its plane) or shared edges at
        # the same distance
        diff = (r32 != ids) & (ids >= 0)
        assert np.all(np.abs(h["t"][diff] - t[diff]) <= 1e-5 * t[diff])
        o32.close()
        f64.close()


CASES = [
    ("cornell, Halton light draws", lambda: scenes.cornell(width=24, height=24, spp=512, max_bounces=5), 1),
    ("cornell, MRG-style light draws", lambda: scenes.cornell(width=24, height=24, spp=512, max_bounces=5), 0),
    ("principled room, roulette from 2", lambda: scenes.principled_room(width=24, height=24, spp=512), 0),
    ("principled room, no roulette", lambda: scenes.principled_room(width=24, height=24, spp=512, rr_start=-1), 0),
    ("principled icospheres, lens", lambda: scenes.icospheres(n_spheres=60, level=2, box=15.0, width=24, height=16,
                                                              spp=512, max_bounces=6, rr_start=3), 0),
]


@pytest.mark.parametrize("name,make,mode", CASES, ids=[c[0] for c in CASES])
def test_fp64_expectation_matches_float_path(name, make, mode):
    from oracle import oracle
    sc = make()
    rd = dict(sc.render, rng_mode=mode)
    cam = dict(sc.camera)
    if "lens" in name:
        cam.update(aperture=0.4, focus_distance=30.0)
    W, H, S, L = rd["width"], rd["height"], rd["spp"], rd["max_bounces"]
    a = oracle.OracleScene(sc, use_bvh=True).render(cam, rd, _pool(S, L, W * H, 5)).astype(np.float64)
    f64 = oracle.F64Scene(sc)
    b, var = f64.render(cam, rd, S, seed=3, with_var=True)
    b2 = f64.render(cam, rd, S, seed=4)
    f64.close()
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert b.mean() > 0.01
    # float path vs fp64, and fp64 vs itself (the same statistic's own spread)
    z = _mean_z(a, b, var, S, S)
    z_self = _mean_z(b2, b, var, S, S)
    assert abs(z) < 4.0, f"{name}: float mean {a.mean():.5f}, fp64 {b.mean():.5f}, z = {z:.2f}"
    assert abs(z_self) < 4.0
    # per row too (16-24 z-scores).  Their mean square is 1 for light-tailed
    # samples; paths whose throughput is clamped to (1, 1, 1) and then escape
    # add the white background (hybrid-pt.cpp:567-572), a rare large sample
    # that the one-sample variance of the reference render underestimates,
    # which lifts it to 2-4 here (the same for fp64 against itself).  A
    # bias would grow it with the sample count.
    rows = [_mean_z(a[r], b[r], var[r], S, S) for r in range(H)]
    assert np.mean(np.square(rows)) < 6.0, rows


def _golden():
    if not GOLDEN.exists():
        pytest.skip("tests/golden/fp64_refs.npz missing")
    return dict(np.load(GOLDEN))


def test_fp64_reference_images_match_their_generators():
    """The committed reference images belong to the current scene generators
    and are converged: finite, non-trivial, thousands of spp."""
    import importlib.util
    g = _golden()
    spec = importlib.util.spec_from_file_location("make_fp64_refs", GOLDEN.parent / "make_fp64_refs.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    for key, sc, rd, (r0, r1), spp, seed in mod.workloads():
        img = g[key]
        assert img.shape == (r1 - r0, rd["width"], 3), key
        assert np.isfinite(img).all() and img.mean() > 0.01, key
        assert int(g[key + "_spp"]) == spp >= 1024, key
        assert tuple(g[key + "_rows"]) == (r0, r1), key
        assert float(g[key + "_check"]) == mod.checksum(sc), f"{key}: scene generator changed; regenerate"
        assert (g[key + "_var"] > 0).all()


def test_float_path_against_fp64_reference_image():
    """The float path (the oracle, which the GPU frames equal bit for bit) on
    the whole Cornell configuration (256x256, 16 spp, 5 bounces, Halton light
    draws), against the committed 4096-spp fp64 image: unbiased (mean within
    4 standard errors) and with the RMSE the noise of 16 + 4096 samples
    predicts."""
    from oracle import oracle
    g = _golden()
    sc = scenes.cornell()
    rd = dict(sc.render)
    W, H, S, L = rd["width"], rd["height"], rd["spp"], rd["max_bounces"]
    a = oracle.OracleScene(sc, use_bvh=False).render(sc.camera, rd, _pool(S, L, H * W, 7))
    ref = g["c0"].astype(np.float64)
    var = np.broadcast_to(g["c0_var"], ref.shape)
    z = _mean_z(a.astype(np.float64), ref, var, S, int(g["c0_spp"]))
    assert abs(z) < 4.0, z
    rmse = np.sqrt(np.mean((a - ref) ** 2))
    expected = np.sqrt(g["c0_var"].mean() * (1.0 / S + 1.0 / int(g["c0_spp"])))
    assert 0.75 < rmse / expected < 1.33, (rmse, expected)


def test_fp64_refuses_what_it_does_not_cover():
    from oracle import oracle
    sc = scenes.icospheres(n_spheres=4, level=1, box=6.0, width=8, height=8, spp=1, max_bounces=2, n_lights=1)
    sky = {"type": gbpt.GB_LIGHT_SKY, "map": scenes.procedural_sky(16, 8), "scale": 1.0, "diameter": 10.0,
           "power": -1.0}
    with_sky = scenes.SceneData(sc.positions, sc.normals, sc.material_index, sc.materials, sc.params,
                                sc.lights + [sky], sc.camera, sc.render)
    with pytest.raises(ValueError):
        oracle.F64Scene(with_sky)
