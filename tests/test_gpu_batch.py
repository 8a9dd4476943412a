"""Batched frames (gb_render_batch): several scenes of uneven sizes, spp,
bounce counts, RNG modes and seeds share one wavefront frame.  Every
scene's image must be bit-identical to gb_render of that scene alone (which
the frame tests pin to the oracle), whether the slot-pool loop runs from the
host or as a CUDA graph with a conditional while node; one member is also
checked against the oracle directly."""
import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu


def _jobs():
    a = scenes.cornell(width=48, height=40, spp=4, max_bounces=5)
    b = scenes.icospheres(n_spheres=40, level=2, box=20.0, width=40, height=30, spp=2, max_bounces=6, rr_start=2)
    c = scenes.cornell(width=32, height=32, spp=6, max_bounces=3)
    d = scenes.icospheres(n_spheres=12, level=3, box=10.0, width=24, height=24, spp=1, max_bounces=4, rr_start=-1,
                          seed_geometry=5)
    return [
        (a, dict(a.camera), dict(a.render, seed=0)),
        (b, dict(b.camera), dict(b.render, seed=7)),
        (c, dict(c.camera, aperture=0.05, focus_distance=1.9), dict(c.render, seed=3)),
        (d, dict(d.camera), dict(d.render, rng_mode=gbpt.GB_RNG_HALTON_LIGHT, seed=11)),
    ]


def _singles(ctx, handles, jobs):
    return [h.render(cam, rd) for h, (_, cam, rd) in zip(handles, jobs)]


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_single_renders(gpu_ctx, graph):
    jobs = _jobs()
    handles = [gpu_ctx.scene(sc) for sc, _, _ in jobs]
    singles = _singles(gpu_ctx, handles, jobs)
    batch = gpu_ctx.render_batch([(h, cam, rd) for h, (_, cam, rd) in zip(handles, jobs)], graph=graph)
    for i, (s, b) in enumerate(zip(singles, batch)):
        assert np.array_equal(s, b), f"scene {i}: max abs diff {np.abs(s - b).max():.3g}"
    st = gpu_ctx.stats()
    assert st["camera_rays"] == sum(rd["width"] * rd["height"] * rd["spp"] for _, _, rd in jobs)
    assert st["paths_done"] == max(rd["spp"] for _, _, rd in jobs)
    for h in handles:
        h.close()


def test_batch_small_pool_and_chunks(gpu_ctx):
    """A slot pool far smaller than the frame and a sample budget that splits
    the rounds into several chunks give the same images."""
    jobs = _jobs()
    handles = [gpu_ctx.scene(sc) for sc, _, _ in jobs]
    ref = gpu_ctx.render_batch([(h, cam, rd) for h, (_, cam, rd) in zip(handles, jobs)], graph=False)
    old = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(slots=333, sample_mb=1)
        for graph in (False, True):
            got = gpu_ctx.render_batch([(h, cam, rd) for h, (_, cam, rd) in zip(handles, jobs)], graph=graph)
            for r, g in zip(ref, got):
                assert np.array_equal(r, g)
    finally:
        gpu_ctx.set_tuning(slots=old["slots"], sample_mb=old["sample_mb"])
    for h in handles:
        h.close()


def test_batch_member_vs_oracle(gpu_ctx):
    from oracle import oracle
    jobs = _jobs()
    handles = [gpu_ctx.scene(sc) for sc, _, _ in jobs]
    batch = gpu_ctx.render_batch([(h, cam, rd) for h, (_, cam, rd) in zip(handles, jobs)], graph=True)
    sc, cam, rd = jobs[1]
    pool = gpu_ctx.mrg_pool(rd["width"] * rd["height"], rd["spp"] * rd["max_bounces"], seed=rd["seed"])
    ref = oracle.OracleScene(sc, use_bvh=True).render(cam, rd, pool)
    diff = np.abs(batch[1].astype(np.float64) - ref)
    assert (diff <= 1e-4 * np.abs(ref) + 1e-6).all()
    for h in handles:
        h.close()


def test_graph_single_render_and_reuse(gpu_ctx):
    """tuning.graph = 2 runs single renders as chunk graphs; a second render
    of the same layout reuses the instantiated graph and repeats the image."""
    sc = scenes.icospheres(n_spheres=30, level=2, box=15.0, width=48, height=32, spp=5, max_bounces=5, rr_start=3)
    h = gpu_ctx.scene(sc)
    loop = h.render(sc.camera, sc.render)
    old = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(graph=2)
        assert gpu_ctx.get_tuning()["graph"] == 2
        g1 = h.render(sc.camera, sc.render)
        g2 = h.render(sc.camera, sc.render)
    finally:
        gpu_ctx.set_tuning(graph=old["graph"])
    assert np.array_equal(loop, g1)
    assert np.array_equal(g1, g2)
    h.close()


def test_batch_errors(gpu_ctx):
    import ctypes as C
    sc = scenes.cornell(width=8, height=8, spp=1, max_bounces=2)
    h = gpu_ctx.scene(sc)
    lib = gpu_ctx.lib
    assert lib.gb_render_batch(gpu_ctx.h, 0, None, 0, 0) == gbpt.GB_ERR_INVALID
    items = (gbpt.BatchItem * 1)()
    items[0] = gbpt.BatchItem(h.h, gbpt.make_camera(sc.camera), gbpt.make_render_desc(sc.render), None)
    assert lib.gb_render_batch(gpu_ctx.h, 1, items, 0, 0) == gbpt.GB_ERR_INVALID  # null output
    other = gbpt.Context(0)
    try:
        out = np.empty((8, 8, 3), np.float32)
        items[0] = gbpt.BatchItem(h.h, gbpt.make_camera(sc.camera), gbpt.make_render_desc(sc.render),
                                  out.ctypes.data_as(C.c_void_p))
        assert lib.gb_render_batch(other.h, 1, items, 0, 0) == gbpt.GB_ERR_INVALID  # scene of another context
    finally:
        other.close()
    # a batch of two cannot be read through the single-scene reader
    out2 = np.empty((8, 8, 3), np.float32)
    items2 = (gbpt.BatchItem * 2)()
    items2[0] = gbpt.BatchItem(h.h, gbpt.make_camera(sc.camera), gbpt.make_render_desc(sc.render),
                               out.ctypes.data_as(C.c_void_p))
    items2[1] = gbpt.BatchItem(h.h, gbpt.make_camera(sc.camera), gbpt.make_render_desc(sc.render),
                               out2.ctypes.data_as(C.c_void_p))
    assert lib.gb_render_batch(gpu_ctx.h, 2, items2, 0, 1) == gbpt.GB_OK
    assert np.array_equal(out, out2)
    assert lib.gb_render_read(gpu_ctx.h, out.ctypes.data_as(C.c_void_p), 0) == gbpt.GB_ERR_INVALID
    h.close()


def test_autotune_keeps_images(gpu_ctx):
    """gb_autotune returns a valid tuning with a positive frame time, leaves
    it set, and the batch renders the same images under it."""
    jobs = _jobs()
    handles = [gpu_ctx.scene(sc) for sc, _, _ in jobs]
    hj = [(h, cam, rd) for h, (_, cam, rd) in zip(handles, jobs)]
    old = gpu_ctx.get_tuning()
    ref = gpu_ctx.render_batch(hj, graph=False)
    try:
        best, ms = gpu_ctx.autotune(hj, proxy_spp=2, repeats=1)
        assert ms > 0.0
        assert best == gpu_ctx.get_tuning()
        assert best["graph"] in (1, 2) and 1 <= best["tri_mode"] <= 4 and 1 <= best["refill"] <= 32
        assert best["stack_depth"] in (24, 32) and best["block_threads"] in (64, 128)
        got = gpu_ctx.render_batch(hj, graph=None)
        for r, g in zip(ref, got):
            assert np.array_equal(r, g)
    finally:
        gpu_ctx.set_tuning(**{k: v for k, v in old.items()})
    for h in handles:
        h.close()
