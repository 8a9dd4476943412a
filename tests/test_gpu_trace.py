"""Traversal parity: GPU closest / any hit vs the CPU oracle (brute force and
its own binary BVH).  Hits are bit-exact: same canonical triangle id, same
t, beta, gamma bits, for every ray (the closest-hit rule is the minimum of
(t, id), which does not depend on the tree)."""
import numpy as np
import pytest

from globillum_gb300 import scenes

pytestmark = pytest.mark.gpu


def _oracle(sc, use_bvh):
    from oracle import oracle
    return oracle.OracleScene(sc, use_bvh=use_bvh)


def _check_closest(g, o):
    assert np.array_equal(g["ref"], o["ref"]), f"{(g['ref'] != o['ref']).sum()} triangle ids differ"
    hit = o["ref"] != 0xFFFFFFFF
    for k in ("t", "beta", "gamma"):
        assert np.array_equal(g[k][hit].view(np.uint32), o[k][hit].view(np.uint32)), k


@pytest.mark.parametrize("use_bvh", [False, True])
def test_cornell_closest_any(gpu_ctx, use_bvh):
    sc = scenes.cornell()
    scene = gpu_ctx.scene(sc)
    orc = _oracle(sc, use_bvh)
    o, d = scenes.random_rays(sc, 50000, seed=3)
    tmax = np.full(o.shape[0], 3.4e38, np.float32)
    _check_closest(scene.trace_closest(o, d, tmax), orc.trace_closest(o, d, tmax))
    tmax2 = np.random.default_rng(4).uniform(0.0, 1.5, o.shape[0]).astype(np.float32)
    _check_closest(scene.trace_closest(o, d, tmax2), orc.trace_closest(o, d, tmax2))
    assert np.array_equal(scene.trace_any(o, d, tmax2), orc.trace_any(o, d, tmax2))
    scene.close()


def test_icospheres_closest_any(gpu_ctx):
    sc = scenes.icospheres(n_spheres=40, level=3, box=20.0)
    scene = gpu_ctx.scene(sc)
    orc = _oracle(sc, True)
    o, d = scenes.random_rays(sc, 100000, seed=5)
    tmax = np.full(o.shape[0], 3.4e38, np.float32)
    g = scene.trace_closest(o, d, tmax)
    _check_closest(g, orc.trace_closest(o, d, tmax))
    assert (g["ref"] != 0xFFFFFFFF).mean() > 0.2
    tm = np.random.default_rng(6).uniform(0.0, 30.0, o.shape[0]).astype(np.float32)
    assert np.array_equal(scene.trace_any(o, d, tm), orc.trace_any(o, d, tm))
    scene.close()


def test_edge_rays(gpu_ctx):
    """Empty batch, negative max_t (no ray), axis-parallel directions, NaN
    rays and origins inside the room."""
    sc = scenes.cornell()
    scene = gpu_ctx.scene(sc)
    orc = _oracle(sc, False)
    empty = np.zeros((0, 3), np.float32)
    assert scene.trace_closest(empty, empty, np.zeros(0, np.float32)).shape == (0,)
    rng = np.random.default_rng(7)
    n = 6000
    o = rng.uniform(0.01, 0.99, size=(n, 3)).astype(np.float32)
    axes = np.eye(3, dtype=np.float32)
    d = np.concatenate([axes, -axes] * (n // 6))
    tmax = np.full(n, 3.4e38, np.float32)
    tmax[::7] = -1.0
    g = scene.trace_closest(o, d, tmax)
    _check_closest(g, orc.trace_closest(o, d, tmax))
    assert (g["ref"][::7] == 0xFFFFFFFF).all()
    # grid-aligned origins on the quad seams (x = 0.5 / z = 0.5 lines)
    o2 = o.copy()
    o2[:, 0] = 0.5
    o2[:, 2] = 0.5
    _check_closest(scene.trace_closest(o2, d, np.full(n, 3.4e38, np.float32)),
                   orc.trace_closest(o2, d, np.full(n, 3.4e38, np.float32)))
    bad = np.full((4, 3), np.nan, np.float32)
    h = scene.trace_closest(bad, bad, np.full(4, 1.0, np.float32))
    assert (h["ref"] == 0xFFFFFFFF).all()
    assert not scene.trace_any(bad, bad, np.full(4, 1.0, np.float32)).any()
    scene.close()
