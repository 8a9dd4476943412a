"""The oracle's FP64 adjoint reference (orc_adjoint_f64, forward-mode dual
numbers in double) against central finite differences of the oracle's own
float frame.  On the Cornell room with Lambert materials, Russian roulette
off and explicit light powers, no random choice depends on an albedo or an
emission: the light pick uses the fixed powers, the cosine-weighted
directions ignore the albedo, and no throughput reaches the clamp (albedo
<= 0.8).  The frame is then a smooth function of those parameters at fixed
pools (polynomial in the albedos, linear in the emission), so the finite
differences of the plain render are its derivative."""
import copy

import numpy as np
import pytest

from globillum_gb300 import scenes
from oracle import oracle


def _scene():
    sc = scenes.cornell(width=24, height=24, spp=2, max_bounces=3)
    for l in sc.lights:  # explicit power: the pick no longer follows the emission
        w, h = l["wh"]
        l["power"] = float(w * h * sum(l["col"]) * 0.333)
    return sc


def _loss(sc, pool, dimg):
    with_scene = oracle.OracleScene(sc, use_bvh=False)
    img = with_scene.render(sc.camera, sc.render, pool).astype(np.float64)
    with_scene.close()
    return float((img * dimg).sum())


def _perturb(sc, idx, h):
    s2 = copy.deepcopy(sc)
    nm = len(s2.materials)
    if idx < 5 * nm:
        m, k = divmod(idx, 5)
        d = list(s2.materials[m]["diffuse"])
        d[k] += h
        s2.materials[m]["diffuse"] = tuple(d)
    else:
        l, c = divmod(idx - 5 * nm, 3)
        col = list(s2.lights[l]["col"])
        col[c] += h
        s2.lights[l]["col"] = tuple(col)
    return s2


@pytest.mark.parametrize("which", ["albedo", "emission"])
def test_fp64_reference_matches_finite_differences(which):
    sc = _scene()
    rd = sc.render
    n = rd["width"] * rd["height"]
    rng = np.random.default_rng(5)
    pool = rng.uniform(1e-6, 1.0, size=(rd["spp"] * rd["max_bounces"], n, 3)).astype(np.float32)
    dimg = rng.normal(size=(rd["height"], rd["width"], 3)).astype(np.float32)
    nm = len(sc.materials)
    sel = [0, 4 * 5 + 1, 6 * 5 + 2, 2 * 5 + 0] if which == "albedo" else [5 * nm + 0, 5 * nm + 1, 5 * nm + 2]
    orc = oracle.OracleScene(sc, use_bvh=False)
    grad = orc.adjoint_f64(sc.camera, rd, pool, dimg, sel)
    orc.close()
    h = 1e-2 if which == "albedo" else 0.5
    for j, idx in enumerate(sel):
        fd = (_loss(_perturb(sc, idx, h), pool, dimg) - _loss(_perturb(sc, idx, -h), pool, dimg)) / (2 * h)
        assert abs(grad[j] - fd) <= 2e-3 * abs(fd) + 1e-4, (idx, grad[j], fd)
        assert abs(grad[j]) > 1e-3  # the parameter matters for this frame


def _metal_scene(spp, mode, background):
    """Principled icospheres with metallic values inside the light-pick
    intervals (not at a boundary, where the expected frame has a kink), no
    roulette."""
    sc = scenes.icospheres(n_spheres=30, level=2, box=10.0, width=16, height=16, spp=spp, max_bounces=4,
                           n_materials=4, n_lights=2, rr_start=-1)
    for i, p in enumerate(sc.params):
        p["metallic"] = (0.3, 0.7, 0.2, 0.8)[i]
        p["roughness"] = 0.3 + 0.1 * i
    sc.render["rng_mode"] = mode
    sc.render["background"] = background
    return sc


def _replay_and_differences(sc, k):
    """FP64 replay gradients with and without the sampling terms, and central
    differences (h = 0.02) of the loss sum(w * frame) on the same 2048-spp
    pools, for parameter k (3 roughness, 4 metallic) of the 4 materials."""
    rd = dict(sc.render)
    W, H, L, S = rd["width"], rd["height"], rd["max_bounces"], rd["spp"]
    pool = np.maximum(np.random.default_rng(1).uniform(0, 1, (S * L, W * H, 3)).astype(np.float32),
                      np.float32(1e-7))
    w = np.random.default_rng(2).uniform(0, 1, (H, W, 3)).astype(np.float32)
    sel = np.array([5 * m + k for m in range(4)], np.int32)
    o = oracle.OracleScene(sc)
    g = o.adjoint_f64(sc.camera, rd, pool, w, sel, sampling_terms=True)
    gf = o.adjoint_f64(sc.camera, rd, pool, w, sel, sampling_terms=False)
    o.close()
    key = "roughness" if k == 3 else "metallic"
    fd = []
    for m in range(4):
        vals = []
        for sgn in (1.0, -1.0):
            s2 = copy.deepcopy(sc)
            s2.params[m][key] += sgn * 0.02
            o2 = oracle.OracleScene(s2, use_bvh=True)
            vals.append(float((o2.render(s2.camera, rd, pool).astype(np.float64) * w).sum()))
            o2.close()
        fd.append((vals[0] - vals[1]) / 0.04)
    return g, gf, np.array(fd)


@pytest.mark.parametrize("mode", [0, 1], ids=["MRG32k3a light draws", "Halton light draws"])
def test_sampling_terms_estimate_the_expected_frame_derivative(mode):
    """With the sampling terms (gb_ctx_set_gradient_terms(ctx, 1)) the FP64
    replay estimates the derivative of the expected frame, which central
    differences of renders at +-h on the same 2048-spp pools measure (they
    change the lobe choices of the paths whose draw lies within h of the
    threshold, and move the sampled directions):
    * metallic (black background): every gradient within 10 % of the
      differences, where the frozen-sampling form, which misses the lobe
      choice, is off by 20-60 %.  The choice's score is taken given the light
      pick that reads the same draw (MRG32k3a light draws) or unconditionally
      (Halton).  With the white background the reference adds to misses of a
      throughput clamped to exactly (1, 1, 1) (hybrid-pt.cpp:567-572), the
      frame also jumps where a change of metallic makes a throughput reach
      the clamp, a discontinuity in the parameter that no sampling term
      covers;
    * roughness (white background, where reflections that escape add it):
      within 20 % in sum, where the frozen form misses nearly all of it."""
    g, gf, fd = _replay_and_differences(_metal_scene(2048, mode, (0.0, 0.0, 0.0)), 4)
    assert np.all(np.abs(g - fd) <= 0.1 * np.abs(fd)), (g, fd)
    assert np.abs(gf - fd).sum() > 3.0 * np.abs(g - fd).sum()
    g, gf, fd = _replay_and_differences(_metal_scene(2048, mode, (1.0, 1.0, 1.0)), 3)
    assert np.abs(g - fd).sum() < 0.2 * np.abs(fd).sum(), (g, fd)
    assert np.abs(gf - fd).sum() > 0.8 * np.abs(fd).sum()
