"""Textures on the host: the mip chain (compute_mipmaps, material.cu:231-275),
sample_bilin_lod (material.h:88-137) against a float32 numpy restatement of
the reference's function, the shared x^2.2 of textured principled colours,
and oracle frames with textures (a white texture leaves a one-bounce
Lambert frame unchanged; a checkerboard changes it)."""
import numpy as np
import pytest

from globillum_gb300 import scenes
from oracle import oracle

f32 = np.float32


def _mips_numpy(img):
    """compute_mipmaps with k::mipmap's integer 2x2 mean (the right column /
    bottom row of an odd level averaged over the texels that exist)."""
    h, w = img.shape[:2]
    mm = int(np.floor(np.log2(min(w, h))))
    levels = [img.astype(np.int64)]
    for _ in range(mm):
        src = levels[-1]
        sh, sw = src.shape[:2]
        th, tw = (sh + 1) // 2, (sw + 1) // 2
        acc = np.zeros((th, tw, 4), np.int64)
        cnt = np.zeros((th, tw, 1), np.int64)
        for dy in (0, 1):
            for dx in (0, 1):
                part = src[dy::2, dx::2]
                acc[:part.shape[0], :part.shape[1]] += part
                cnt[:part.shape[0], :part.shape[1]] += 1
        levels.append(acc // cnt)
    return np.concatenate([l.reshape(-1, 4) for l in levels]).astype(np.uint8), mm


@pytest.mark.parametrize("shape", [(64, 64), (32, 16), (17, 9), (1, 1), (5, 12)])
def test_mip_chain(shape):
    img = np.random.default_rng(1).integers(0, 256, size=shape + (4,), dtype=np.uint8)
    chain, mm, size = oracle.mipmaps(img)
    ref, mm_ref = _mips_numpy(img)
    assert mm == mm_ref
    assert np.array_equal(chain[:ref.shape[0]], ref)
    assert size == ref.shape[0] + shape[1] + 1 and not chain[ref.shape[0]:].any()  # zero tail


def _sample_numpy(chain, w, h, mm, s, t, diff):
    """sample_bilin_lod in float32, lod from log2 (material.h:88-137)."""
    W, H = w, h
    with np.errstate(divide="ignore", invalid="ignore"):
        lod = f32(np.log2(np.float64(f32(diff) * f32(max(w, h)))))
    lod = f32(mm) if np.isnan(lod) else min(lod, f32(mm))  # fminf(NaN, mm) = mm
    offset, i = 0, 0
    while i < lod:
        offset += W * H
        W, H = (W + 1) // 2, (H + 1) // 2
        i += 1
    s, t = f32(s), f32(t)
    if s < 0:
        s = f32(s + f32(-np.trunc(s) + 1))
    if s >= 1:
        s = f32(s - np.trunc(s))
    if t < 0:
        t = f32(t + f32(-np.trunc(t) + 1))
    if t >= 1:
        t = f32(t - np.trunc(t))
    x, y = f32(s * f32(W)), f32(f32(1 - t) * f32(H))
    nx, ny = int(x), int(y)
    ox = nx - 1 if x - np.floor(x) < 0.5 else nx + 1
    oy = ny - 1 if y - np.floor(y) < 0.5 else ny + 1
    wx, wy = abs(f32(f32(ox) + f32(0.5)) - x), abs(f32(f32(oy) + f32(0.5)) - y)
    ox = ox - W if ox > W else ox + W if ox < 0 else ox
    oy = oy - H if oy > H else oy + H if oy < 0 else oy

    def tx(i):
        return chain[offset + i, :3].astype(np.float32) / f32(255)
    a00, a01 = tx(ny * W + nx), tx(ny * W + ox)
    a10, a11 = tx(oy * W + nx), tx(oy * W + ox)
    a0x = wx * a00 + (f32(1) - wx) * a01
    a1x = wx * a10 + (f32(1) - wx) * a11
    return wy * a0x + (f32(1) - wy) * a1x


@pytest.mark.parametrize("shape", [(64, 64), (48, 20)])
def test_sample_bilin_lod(shape):
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, size=shape + (4,), dtype=np.uint8)
    n = 3000
    s = rng.uniform(-2.5, 3.5, n).astype(np.float32)
    t = rng.uniform(-2.5, 3.5, n).astype(np.float32)
    s[:4] = [0.0, 0.9999999, -1.0, 0.5]
    t[:4] = [0.0, 1.0, 0.0, 1e-9]   # t = 0 reads the row after the level
    diff = np.exp(rng.uniform(np.log(1e-4), np.log(2.0), n)).astype(np.float32)
    diff[:8] = [0.0, np.nan, np.inf, 1e-30, 1.0 / 64, 1.0, 100.0, 0.015]
    got = oracle.tex_sample(img, s, t, diff)
    chain, mm, _ = oracle.mipmaps(img)
    h, w = shape
    ref = np.array([_sample_numpy(chain, w, h, mm, s[i], t[i], diff[i]) for i in range(n)])
    assert np.array_equal(got, ref), np.argwhere((got != ref).any(axis=1))[:5].ravel()


def test_pow22_matches_pow():
    x = np.concatenate([np.random.default_rng(3).uniform(0, 1, 100000), [0.0, 1.0, 1e-30, 0.5, 2.0]])
    got = oracle.pow22(x)
    ref = np.power(x, 2.2)
    assert np.all(np.abs(got - ref) <= 1e-14 * ref + 1e-300)
    same = (got.astype(np.float32) == ref.astype(np.float32)).mean()
    assert same > 0.9999
    assert np.isnan(oracle.pow22(np.array([-0.5, np.nan]))).all()


def _frame(sc, pool_seed=4):
    rd = dict(sc.render, rng_mode=0)
    n = rd["width"] * rd["height"]
    pool = np.random.default_rng(pool_seed).uniform(1e-6, 1, size=(rd["spp"] * rd["max_bounces"], n, 3)).astype(
        np.float32)
    return oracle.OracleScene(sc, use_bvh=False).render(sc.camera, rd, pool)


def test_oracle_frames_with_textures():
    # one bounce at 96 x 64: camera footprints of a few texels only.  A
    # white texture then scales the colours by a bilinear blend of 1.0s,
    # which is exactly 1 (weights in [0.5, 1]).  Deeper bounces are not
    # compared: there the right differential keeps its camera direction (as
    # in the reference), footprints grow until the coarsest level, whose
    # neighbour reads fall past the chain (into the zero tail here, into
    # unset memory in the reference).
    sc = scenes.cornell(width=96, height=64, spp=1, max_bounces=1)
    base = _frame(sc)
    white = scenes.with_textures(sc, fraction=1.0)
    white.textures = [np.full_like(t, 255) for t in white.textures]
    close = np.isclose(_frame(white), base, rtol=1e-5, atol=1e-7).all(axis=2)
    assert close.mean() > 0.99
    sc = scenes.cornell(width=24, height=16, spp=2, max_bounces=3)
    base = _frame(sc)
    tex = scenes.with_textures(sc, fraction=1.0, scale=3.0)
    img = _frame(tex)
    assert np.isfinite(img).all() and not np.array_equal(img, base)
