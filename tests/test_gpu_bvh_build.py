"""Device BVH construction (gb_scene_create_ex with GB_BVH_DEVICE_PLOC) and
refits (gb_scene_refit).  The closest hit is the minimum (t, id) whatever
the tree, so a device-built scene must give the oracle's brute-force hits
and frames bit for bit, like the host-built one; the tests also bound the
traversal cost of the device tree against the host binned-SAH tree."""
import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu


def _oracle(sc, use_bvh=False):
    from oracle import oracle
    return oracle.OracleScene(sc, use_bvh=use_bvh)


def _same_hits(g, o):
    assert np.array_equal(g["ref"], o["ref"]), f"{(g['ref'] != o['ref']).sum()} triangle ids differ"
    hit = o["ref"] != 0xFFFFFFFF
    for k in ("t", "beta", "gamma"):
        assert np.array_equal(g[k][hit].view(np.uint32), o[k][hit].view(np.uint32)), k


def _frame_and_ref(ctx, sc, rd, scene):
    npx = rd["width"] * rd["height"]
    img = scene.render(sc.camera, rd)
    pool = ctx.mrg_pool(npx, rd["spp"] * rd["max_bounces"], seed=rd.get("seed", 0))
    ref = _oracle(sc).render(sc.camera, rd, pool)
    return img, ref


@pytest.mark.parametrize("radius", [1, 16, 32])
def test_device_tree_hits_match_oracle(gpu_ctx, radius):
    sc = scenes.icospheres(n_spheres=40, level=3, box=20.0)
    scene = gpu_ctx.scene(sc, builder="device", ploc_radius=radius)
    info = scene.info()
    assert info["builder"] == gbpt.GB_BVH_DEVICE_PLOC and info["build_passes"] > 0
    assert info["binary_nodes"] == 2 * info["num_triangles"] - 1 and 1 <= info["depth"] <= 32
    orc = _oracle(sc)
    o, d = scenes.random_rays(sc, 100000, seed=5)
    tmax = np.full(o.shape[0], 3.4e38, np.float32)
    g = scene.trace_closest(o, d, tmax)
    _same_hits(g, orc.trace_closest(o, d, tmax))
    assert (g["ref"] != 0xFFFFFFFF).mean() > 0.2
    tm = np.random.default_rng(6).uniform(0.0, 30.0, o.shape[0]).astype(np.float32)
    assert np.array_equal(scene.trace_any(o, d, tm), orc.trace_any(o, d, tm))
    scene.close()


def test_device_tree_frame_bit_exact(gpu_ctx):
    sc = scenes.icospheres(n_spheres=12, level=2, box=10.0, width=48, height=32, spp=4, max_bounces=4, n_lights=2)
    rd = dict(sc.render)
    dev = gpu_ctx.scene(sc, builder="device")
    img, ref = _frame_and_ref(gpu_ctx, sc, rd, dev)
    host = gpu_ctx.scene(sc)
    assert np.array_equal(img, host.render(sc.camera, rd))
    assert np.array_equal(img, ref.astype(np.float32)), np.abs(img - ref).max()
    dev.close()
    host.close()


def test_device_tree_is_deterministic(gpu_ctx):
    sc = scenes.icospheres(n_spheres=30, level=3, box=15.0)
    infos = []
    for _ in range(2):
        s = gpu_ctx.scene(sc, builder="device")
        infos.append({k: v for k, v in s.info().items() if k != "build_ms"})
        s.close()
    assert infos[0] == infos[1]


def _tiny(tris):
    pos = np.asarray(tris, np.float32).reshape(-1, 9)
    n = pos.shape[0]
    return scenes.SceneData(positions=pos, normals=None, material_index=np.zeros(n, np.int32),
                            materials=[{"diffuse": (0.5, 0.5, 0.5), "principled": -1}], params=[],
                            lights=[], camera={}, render={})


@pytest.mark.parametrize("n", [1, 2, 3, 4, 9, 64])
def test_small_and_degenerate_inputs(gpu_ctx, n):
    """1 .. 64 triangles, including identical copies (equal Morton codes and
    boxes, so every pair ties)."""
    rng = np.random.default_rng(n)
    base = rng.uniform(-1, 1, (n, 9)).astype(np.float32)
    for tris in (base, np.repeat(base[:1], n, axis=0)):
        sd = _tiny(tris)
        s = gpu_ctx.scene(sd, builder="device")
        assert s.info()["num_triangles"] == n
        o = rng.uniform(-2, 2, (4000, 3)).astype(np.float32)
        d = (rng.uniform(-1, 1, (4000, 3)) - o * 0.3).astype(np.float32)
        tmax = np.full(4000, 3.4e38, np.float32)
        _same_hits(s.trace_closest(o, d, tmax), _oracle(sd).trace_closest(o, d, tmax))
        s.close()


def test_device_build_rejects_bad_input(gpu_ctx):
    sc = scenes.cornell()
    bad = sc.positions.copy()
    bad[3, 4] = np.nan
    with pytest.raises(gbpt.GBError, match="non-finite"):
        gpu_ctx.scene(scenes.SceneData(**{**sc.__dict__, "positions": bad}), builder="device")
    with pytest.raises(gbpt.GBError, match="radius"):
        gpu_ctx.scene(sc, builder="device", ploc_radius=33)


def test_refit_moved_vertices(gpu_ctx):
    sc = scenes.icospheres(n_spheres=12, level=2, box=10.0, width=40, height=30, spp=2, max_bounces=3, n_lights=2)
    rd = dict(sc.render)
    s = gpu_ctx.scene(sc, builder="device")
    before = s.info()
    # every sphere's vertices pushed along a smooth field: boxes change, topology kept
    p = sc.positions.reshape(-1, 3).astype(np.float64)
    moved = (p + 0.4 * np.sin(p[:, [1, 2, 0]] * 0.7)).astype(np.float32).reshape(-1, 9)
    sm = scenes.SceneData(**{**sc.__dict__, "positions": moved, "normals": None})
    s.refit(moved)
    assert {k: v for k, v in s.info().items() if k != "build_ms"} == \
        {k: v for k, v in before.items() if k != "build_ms"}
    orc = _oracle(sm)
    o, d = scenes.random_rays(sm, 50000, seed=8)
    tmax = np.full(o.shape[0], 3.4e38, np.float32)
    _same_hits(s.trace_closest(o, d, tmax), orc.trace_closest(o, d, tmax))
    img, ref = _frame_and_ref(gpu_ctx, sm, rd, s)
    assert np.array_equal(img, ref.astype(np.float32)), np.abs(img - ref).max()
    # a rejected refit leaves the scene as it was
    bad = moved.copy()
    bad[0, 0] = np.inf
    with pytest.raises(gbpt.GBError, match="non-finite"):
        s.refit(bad)
    assert np.array_equal(s.render(sm.camera, rd), img)
    s.close()
    h = gpu_ctx.scene(sc)
    with pytest.raises(gbpt.GBError) as ei:
        h.refit(moved)
    assert ei.value.code == gbpt.GB_ERR_UNSUPPORTED
    h.close()


def test_device_tree_traversal_cost(gpu_ctx):
    """Node visits and triangle tests per ray of the device tree stay within
    1.3x of the host binned-SAH tree on the same rays."""
    sc = scenes.icospheres(n_spheres=200, level=3, box=40.0, width=128, height=96, spp=2, max_bounces=4)
    rd = dict(sc.render)
    cost = {}
    for b in ("host", "device"):
        s = gpu_ctx.scene(sc, builder=b)
        s.render(sc.camera, rd, instrumented=True)
        st = gpu_ctx.stats()
        rays = st["camera_rays"] + st["extension_rays"]
        cost[b] = (st["closest_node_visits"] + st["closest_tri_tests"]) / rays
        s.close()
    assert cost["device"] <= 1.3 * cost["host"], cost


@pytest.mark.parametrize("builder,prim_cost", [("host", 0.0), ("host", 1.0), ("device", 0.0), ("device", 2.0)])
def test_sah_wide_collapse_hits_and_frame(gpu_ctx, builder, prim_cost):
    """The SAH-optimal 8-wide grouping (wide_collapse 1, the default) of
    either builder's tree gives the oracle's hits and frame, with fewer nodes
    than the greedy grouping (wide_collapse 2) of the same builder."""
    sc = scenes.icospheres(n_spheres=12, level=2, box=10.0, width=48, height=32, spp=3, max_bounces=4, n_lights=2)
    s = gpu_ctx.scene(sc, builder=builder, wide_collapse=1, prim_cost=prim_cost)
    g = gpu_ctx.scene(sc, builder=builder, wide_collapse=2)
    assert s.info()["num_nodes"] < g.info()["num_nodes"]
    orc = _oracle(sc)
    o, d = scenes.random_rays(sc, 50000, seed=9)
    tmax = np.full(o.shape[0], 3.4e38, np.float32)
    _same_hits(s.trace_closest(o, d, tmax), orc.trace_closest(o, d, tmax))
    img, ref = _frame_and_ref(gpu_ctx, sc, dict(sc.render), s)
    assert np.array_equal(img, ref.astype(np.float32))
    s.close()
    g.close()
    with pytest.raises(gbpt.GBError, match="wide_collapse"):
        gpu_ctx.scene(sc, wide_collapse=3)
