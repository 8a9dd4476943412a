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
