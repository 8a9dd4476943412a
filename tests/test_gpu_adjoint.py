"""Path-replay adjoint (gb_forward / gb_backward) on the GPU.

Checks: the frozen-sampling forward at the current parameters is the plain
frame bit for bit; the adjoint gradient agrees with the oracle's FP64
dual-number replay of the same paths, and with central finite differences
(h = 1e-3) of gb_forward(eval_params) at common random numbers; batched
backward equals per-scene backward; parameters round-trip; and a
torch.autograd.Function built on the pair (defined here, in the test
harness only) drives a short inverse-rendering loop downhill."""
import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes

pytestmark = pytest.mark.gpu


def _scene(seed=7, w=48, h=32, spp=4, bounces=4, rr=3):
    return scenes.icospheres(n_spheres=24, level=2, box=12.0, width=w, height=h, spp=spp, max_bounces=bounces,
                             n_materials=16, n_lights=2, seed_geometry=seed, seed_materials=seed + 1,
                             seed_lights=seed + 2, rr_start=rr)


def _visible_params(grad, n_mats, k, rng):
    """k parameters with clearly nonzero gradient (materials and lights)."""
    cand = np.flatnonzero(np.abs(grad) > 1e-3 * np.abs(grad).max())
    return np.sort(rng.choice(cand, size=min(k, cand.size), replace=False))


def test_params_round_trip(gpu_ctx):
    sc = _scene()
    s = gpu_ctx.scene(sc)
    x = s.get_params()
    assert x.shape == (5 * len(sc.materials) + 3 * len(sc.lights),)
    img0 = s.render(sc.camera, sc.render)
    x2 = x.copy()
    x2[0:3] *= 0.5
    x2[-3:] *= 2.0
    s.set_params(x2)
    assert np.array_equal(s.get_params(), x2)
    img1 = s.render(sc.camera, sc.render)
    assert not np.array_equal(img0, img1)
    s.set_params(x)
    assert np.array_equal(s.render(sc.camera, sc.render), img0)
    s.close()


def test_frozen_forward_at_current_params_is_the_frame(gpu_ctx):
    sc = _scene()
    s = gpu_ctx.scene(sc)
    img = s.render(sc.camera, sc.render)
    rep = s.forward(sc.camera, sc.render, eval_params=s.get_params())
    assert np.array_equal(img, rep)
    s.close()


def test_backward_matches_fp64_replay(gpu_ctx):
    from oracle import oracle
    sc = _scene()
    rd = sc.render
    s = gpu_ctx.scene(sc)
    rng = np.random.default_rng(1)
    dimg = rng.normal(size=(rd["height"], rd["width"], 3)).astype(np.float32)
    grad = s.backward(sc.camera, rd, dimg)
    assert np.isfinite(grad).all() and np.abs(grad).max() > 0
    sel = _visible_params(grad, len(sc.materials), 32, rng)
    pool = gpu_ctx.mrg_pool(rd["width"] * rd["height"], rd["spp"] * rd["max_bounces"], seed=rd["seed"])
    orc = oracle.OracleScene(sc, use_bvh=True)
    ref = orc.adjoint_f64(sc.camera, rd, pool, dimg, sel)
    orc.close()
    scale = np.abs(ref).max()
    err = np.abs(grad[sel].astype(np.float64) - ref)
    assert (err <= 1e-3 * np.abs(ref) + 1e-5 * scale).all(), (sel[np.argmax(err)], err.max(), scale)
    s.close()


def test_backward_with_sampling_terms_matches_fp64_replay(gpu_ctx):
    """gb_ctx_set_gradient_terms(ctx, 1): the device sweep with the
    derivatives of the sampling decisions (metallic lobe choice, GTR2
    half-vector density and Walter weight in roughness) against the oracle's
    FP64 replay with the same terms, on the same MRG32k3a pools, for both
    light-draw modes; the frozen gradient must differ from it."""
    from oracle import oracle
    sc = _scene(seed=9)
    for mode in (gbpt.GB_RNG_MRG32K3A_POOL, gbpt.GB_RNG_HALTON_LIGHT):
        rd = dict(sc.render, rng_mode=mode)
        s = gpu_ctx.scene(sc)
        rng = np.random.default_rng(3)
        dimg = rng.normal(size=(rd["height"], rd["width"], 3)).astype(np.float32)
        frozen = s.backward(sc.camera, rd, dimg)
        gpu_ctx.set_gradient_terms(True)
        try:
            grad = s.backward(sc.camera, rd, dimg)
        finally:
            gpu_ctx.set_gradient_terms(False)
        assert np.isfinite(grad).all()
        nm = len(sc.materials)
        rough_metal = np.array([5 * m + k for m in range(nm) for k in (3, 4)])
        sel = np.union1d(_visible_params(grad, nm, 24, rng), rough_metal)
        pool = gpu_ctx.mrg_pool(rd["width"] * rd["height"], rd["spp"] * rd["max_bounces"], seed=rd["seed"])
        orc = oracle.OracleScene(sc, use_bvh=True)
        ref = orc.adjoint_f64(sc.camera, rd, pool, dimg, sel, sampling_terms=True)
        orc.close()
        scale = np.abs(ref).max()
        err = np.abs(grad[sel].astype(np.float64) - ref)
        assert (err <= 2e-3 * np.abs(ref) + 2e-5 * scale).all(), (mode, sel[np.argmax(err)], err.max(), scale)
        # the sampling terms moved the roughness and metallic gradients of
        # the principled metals (Lambert and glass materials keep theirs)
        moved = np.abs(grad[rough_metal] - frozen[rough_metal]) > 1e-2 * np.abs(grad[rough_metal]).max()
        assert moved.sum() >= 4, moved
        others = np.setdiff1d(np.arange(grad.size), rough_metal)
        assert np.allclose(grad[others], frozen[others], rtol=1e-4, atol=1e-6 * np.abs(frozen).max())
        s.close()


def test_backward_matches_finite_differences(gpu_ctx):
    """L2 loss to a target rendered with other materials; central
    differences of the frozen-sampling forward.  A path whose throughput
    sits at the clamp kink within +-h makes a parameter's difference
    quotient differ from the derivative; errors are therefore judged
    against the gradient scale as well."""
    sc = _scene(seed=11)
    rd = sc.render
    s = gpu_ctx.scene(sc)
    x0 = s.get_params()
    xt = x0.copy()
    nm = len(sc.materials)
    rng = np.random.default_rng(2)
    xt[:5 * nm] = np.clip(x0[:5 * nm] + rng.uniform(-0.3, 0.3, 5 * nm), 0.0, 1.0).astype(np.float32)
    s.set_params(xt)
    target = s.render(sc.camera, rd).astype(np.float64)
    s.set_params(x0)
    img = s.render(sc.camera, rd)
    dimg = (2.0 * (img - target)).astype(np.float32)
    grad = s.backward(sc.camera, rd, dimg)
    sel = _visible_params(grad, nm, 16, rng)
    h = 1e-3
    loss = lambda im: float(((im.astype(np.float64) - target) ** 2).sum())
    rows = []
    for i in sel:
        xp, xm = x0.copy(), x0.copy()
        xp[i] += h
        xm[i] -= h
        fd = (loss(s.forward(sc.camera, rd, xp)) - loss(s.forward(sc.camera, rd, xm))) / (2 * h)
        rows.append((int(i), float(grad[i]), fd))
    g = np.array([r[1] for r in rows])
    fd = np.array([r[2] for r in rows])
    rel = np.abs(g - fd) / np.abs(fd)
    scaled = np.abs(g - fd) / np.abs(grad).max()
    assert np.median(rel) < 1e-3 and scaled.max() < 1e-3, rows
    s.close()


def _plain_differences(s, sc, rd, x0, w, sel, h):
    """Central differences of sum(w * frame) of the plain frame (gb_render
    after gb_scene_set_params: every random number the same, every sampling
    decision re-made) at steps h and h / 2."""
    loss = lambda: float((s.render(sc.camera, rd).astype(np.float64) * w).sum())
    out = []
    for hh in (h, 0.5 * h):
        d = []
        for i in sel:
            xp, xm = x0.copy(), x0.copy()
            xp[i] += hh
            xm[i] -= hh
            s.set_params(xp)
            lp = loss()
            s.set_params(xm)
            d.append((lp - loss()) / (2 * hh))
        out.append(np.array(d))
    s.set_params(x0)
    return out


def test_backward_matches_plain_frame_differences(gpu_ctx):
    """The gradient against central differences of the plain frame at common
    random numbers, relative error <= 1e-3 for each parameter.
    * Lambert room (Halton light draws, no roulette, one light): the frame
      is a polynomial in every albedo and the light colour (brdf / pdf =
      albedo < 1 never reaches the throughput clamp, no sampling decision
      depends on them), so every parameter with a gradient is checked.
    * Principled icospheres (black background, no roulette): colours and
      light colours.  A throughput reaching the clamp, or a sampling decision
      that a colour moves, puts a kink or a jump in the frame; parameters
      whose differences at h and h / 2 disagree by more than 1e-4 are not
      smooth at that scale and are skipped; most must qualify."""
    sc = scenes.cornell(width=32, height=32, spp=4, max_bounces=5)
    rd = sc.render
    s = gpu_ctx.scene(sc)
    x0 = s.get_params()
    w = np.random.default_rng(5).uniform(0.0, 1.0, (rd["height"], rd["width"], 3))
    grad = s.backward(sc.camera, rd, w.astype(np.float32)).astype(np.float64)
    nm = len(sc.materials)
    sel = np.array([5 * m + c for m in range(nm) for c in range(3)] + [5 * nm + c for c in range(3)])
    sel = sel[np.abs(grad[sel]) > 1e-6 * np.abs(grad).max()]
    assert sel.size >= 18
    d1, d2 = _plain_differences(s, sc, rd, x0, w, sel, 1e-3)
    rel = np.abs(grad[sel] - d2) / np.abs(d2)
    assert rel.max() <= 1e-3, (sel[np.argmax(rel)], rel.max())
    s.close()

    sc = _scene(seed=11, rr=-1)
    rd = dict(sc.render, background=(0.0, 0.0, 0.0))
    s = gpu_ctx.scene(sc)
    x0 = s.get_params()
    w = np.random.default_rng(6).uniform(0.0, 1.0, (rd["height"], rd["width"], 3))
    grad = s.backward(sc.camera, rd, w.astype(np.float32)).astype(np.float64)
    nm, nl = len(sc.materials), len(sc.lights)
    sel = np.array([5 * m + c for m in range(nm) for c in range(3)] + [5 * nm + c for c in range(3 * nl)])
    sel = sel[np.abs(grad[sel]) > 1e-3 * np.abs(grad).max()]
    d1, d2 = _plain_differences(s, sc, rd, x0, w, sel, 1e-3)
    smooth = np.abs(d1 - d2) <= 1e-4 * np.abs(d2)
    assert smooth.mean() >= 0.6, (smooth.sum(), sel.size)
    rel = np.abs(grad[sel] - d2) / np.abs(d2)
    assert rel[smooth].max() <= 1e-3, (sel[smooth][np.argmax(rel[smooth])], rel[smooth].max())
    s.close()


def test_backward_batch_equals_single(gpu_ctx):
    """Three scenes of different sizes, spp, bounces and materials (principled
    and Lambert): the batched adjoint, host-driven and as one CUDA graph,
    gives each scene's single gb_backward gradient."""
    c = scenes.cornell(width=32, height=20, spp=2, max_bounces=4)
    c.render["rng_mode"] = gbpt.GB_RNG_MRG32K3A_POOL
    scs = [_scene(seed=3, w=40, h=24, spp=3), _scene(seed=5, w=24, h=24, spp=5, bounces=3), c]
    hs = [gpu_ctx.scene(sc) for sc in scs]
    rng = np.random.default_rng(4)
    gs = [rng.normal(size=(sc.render["height"], sc.render["width"], 3)).astype(np.float32) for sc in scs]
    single = [h.backward(sc.camera, sc.render, g) for h, sc, g in zip(hs, scs, gs)]
    jobs = [(h, sc.camera, sc.render) for h, sc in zip(hs, scs)]
    for graph in (False, True):
        batch = gpu_ctx.backward_batch(jobs, gs, graph=graph)
        for x, y in zip(single, batch):
            assert np.allclose(x, y, rtol=1e-4, atol=1e-6 * np.abs(x).max())
    for h in hs:
        h.close()


def test_backward_rejects_long_paths(gpu_ctx):
    sc = _scene(bounces=17)
    s = gpu_ctx.scene(sc)
    with pytest.raises(gbpt.GBError):
        s.backward(sc.camera, sc.render, np.zeros((32, 48, 3), np.float32))
    s.close()


def test_autograd_inverse_rendering_descends(gpu_ctx):
    torch = pytest.importorskip("torch")
    sc = _scene(seed=13, w=32, h=32, spp=4, bounces=3)
    rd = sc.render
    s = gpu_ctx.scene(sc)
    x_true = s.get_params()
    target = torch.from_numpy(s.render(sc.camera, rd))
    nm = len(sc.materials)

    class Render(torch.autograd.Function):
        """gb_forward / gb_backward as an autograd node (test harness only)."""

        @staticmethod
        def forward(ctx, x):
            s.set_params(x.detach().cpu().numpy())
            return torch.from_numpy(s.render(sc.camera, rd))

        @staticmethod
        def backward(ctx, gimg):
            return torch.from_numpy(s.backward(sc.camera, rd, gimg.contiguous().cpu().numpy()))

    x0 = x_true.copy()
    colour = np.zeros_like(x0, bool)
    for m in range(nm):
        colour[5 * m:5 * m + 3] = True
    x0[colour] = np.clip(x0[colour] * 0.5 + 0.2, 0.0, 1.0)
    x = torch.tensor(x0, requires_grad=True)
    mask = torch.from_numpy(colour.astype(np.float32))
    lo = torch.from_numpy(np.where(colour, 0.0, -np.inf).astype(np.float32))
    hi = torch.from_numpy(np.where(colour, 1.0, np.inf).astype(np.float32))
    opt = torch.optim.Adam([x], lr=2e-2)
    losses = []
    for _ in range(15):
        opt.zero_grad()
        loss = ((Render.apply(x) - target) ** 2).sum()
        loss.backward()
        x.grad *= mask  # only base colours are free
        opt.step()
        with torch.no_grad():
            x.copy_(torch.maximum(torch.minimum(x, hi), lo))  # base colours stay in [0, 1]
        losses.append(loss.item())
    assert losses[-1] < 0.5 * losses[0], losses
    s.set_params(x_true)
    s.close()


def test_fit_step_is_one_graph_and_matches_the_separate_calls(gpu_ctx):
    """gb_fit_step (parameter upload, batched forward frame, L2 loss and
    image gradient on the device, batched adjoint, gradient reduction: one
    CUDA graph launch) gives the batched frame bit for bit, the L2 losses,
    and the gradients of gb_backward_batch fed with 2 (image - target);
    over several steps with changing parameters, and again after another
    render on the context forced the graph to be captured anew."""
    import torch
    scs = [_scene(seed=7), _scene(seed=11, w=40, h=40, spp=3, bounces=3),
           scenes.cornell(width=32, height=24, spp=2, max_bounces=4)]
    scs[2].render["rng_mode"] = gbpt.GB_RNG_MRG32K3A_POOL
    hs = [gpu_ctx.scene(sc) for sc in scs]
    jobs = [(h, sc.camera, sc.render) for h, sc in zip(hs, scs)]
    x0 = [h.get_params() for h in hs]
    rng = np.random.default_rng(3)
    targets = []
    for h, sc, x in zip(hs, scs, x0):
        xt = x.copy()
        nm = 5 * len(sc.materials)
        xt[:nm] = np.clip(xt[:nm] + rng.normal(0.0, 0.1, nm), 0.0, 1.0).astype(np.float32)
        h.set_params(xt)
        targets.append(torch.from_numpy(h.render(sc.camera, sc.render)).cuda())
        h.set_params(x)
    images = [torch.empty_like(t) for t in targets]
    gpu_ctx.fit_prepare(jobs, [t.data_ptr() for t in targets], [i.data_ptr() for i in images])
    xs = [x.copy() for x in x0]
    for step in range(3):
        if step == 2:
            # another render on the context (a larger frame) moves its buffers
            big = scenes.icospheres(n_spheres=8, level=2, box=8.0, width=200, height=150, spp=1, max_bounces=2)
            hb = gpu_ctx.scene(big)
            hb.render(big.camera, big.render)
            hb.close()
        grads, loss = gpu_ctx.fit_step(xs)
        for h, x in zip(hs, xs):
            assert np.array_equal(h.get_params(), x)
        ref = gpu_ctx.render_batch(jobs, graph=True)
        dimgs = []
        for i, (r, t) in enumerate(zip(ref, targets)):
            got = images[i].cpu().numpy()
            assert np.array_equal(got, r), f"step {step} scene {i}: frame differs"
            tn = t.cpu().numpy()
            d = r.astype(np.float64) - tn
            assert np.isclose(loss[i], float((d * d).sum()), rtol=1e-6, atol=0.0)
            dimgs.append((2.0 * (r - tn)).astype(np.float32))
        gref = gpu_ctx.backward_batch(jobs, dimgs, graph=True)
        for g, gr in zip(grads, gref):
            assert np.allclose(g, gr, rtol=1e-4, atol=1e-6 * np.abs(gr).max())
        xs = [np.clip(x - 1e-3 * g / max(1e-12, np.abs(g).max()), 0.0, 1.0).astype(np.float32)
              for x, g in zip(xs, grads)]
        # lights keep their emission (only the materials move)
        for x, x_init, sc in zip(xs, x0, scs):
            x[5 * len(sc.materials):] = x_init[5 * len(sc.materials):]
    for h in hs:
        h.close()


def test_fit_step_of_one_scene_on_a_fresh_context():
    """A fitting step of a single scene on a new context: the frame of one
    scene gives the traversal launches its persisting L2 window, whose
    set-aside the context has not asked for yet when the step is captured.
    The step must still equal gb_render + gb_backward of 2 (image - target)."""
    import torch
    ctx = gbpt.Context(0)
    try:
        sc = _scene(seed=17, w=40, h=32, spp=2, bounces=3)
        h = ctx.scene(sc)
        x0 = h.get_params()
        xt = x0.copy()
        nm = 5 * len(sc.materials)
        xt[:nm] = np.clip(xt[:nm] * 0.8 + 0.1, 0.0, 1.0).astype(np.float32)
        h.set_params(xt)
        target = torch.from_numpy(h.render(sc.camera, sc.render)).cuda()
        h.set_params(x0)
        image = torch.empty_like(target)
        ctx.fit_prepare([(h, sc.camera, sc.render)], [target.data_ptr()], [image.data_ptr()])
        for _ in range(2):
            grads, loss = ctx.fit_step([x0])
            ref = h.render(sc.camera, sc.render)
            assert np.array_equal(image.cpu().numpy(), ref)
            tn = target.cpu().numpy()
            assert np.isclose(loss[0], float(((ref.astype(np.float64) - tn) ** 2).sum()), rtol=1e-6, atol=0.0)
            gref = h.backward(sc.camera, sc.render, (2.0 * (ref - tn)).astype(np.float32))
            assert np.allclose(grads[0], gref, rtol=1e-4, atol=1e-6 * np.abs(gref).max())
        h.close()
    finally:
        ctx.close()


def test_backward_with_a_small_slot_pool(gpu_ctx):
    """Fewer slots than paths (the adjoint's chunks are capped to bound its
    vertex records): the paths replay in several waves of the pool and the
    gradient equals the one of a pool holding every path (sums in another
    order: relative 1e-4)."""
    sc = _scene(seed=21)
    rd = sc.render
    s = gpu_ctx.scene(sc)
    g = np.random.default_rng(8).normal(size=(rd["height"], rd["width"], 3)).astype(np.float32)
    full = s.backward(sc.camera, rd, g)
    old = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(slots=1000)
        small = s.backward(sc.camera, rd, g)
    finally:
        gpu_ctx.set_tuning(slots=old["slots"])
    assert np.allclose(small, full, rtol=1e-4, atol=1e-6 * np.abs(full).max())
    s.close()
