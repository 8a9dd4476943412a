"""Sky light on the host: the shared atan2 / acos used for texel lookup, the
Distribution1D tables and sampling (lights.h:18-60) against a numpy
restatement, and an oracle frame with a sky light (open scene, so misses
and sky NEE samples both contribute)."""
import numpy as np

from globillum_gb300 import scenes
from oracle import oracle


def test_atan2_acos_accuracy():
    rng = np.random.default_rng(0)
    y = rng.uniform(-3, 3, 20000).astype(np.float32)
    x = rng.uniform(-3, 3, 20000).astype(np.float32)
    y[:8] = [0, 0, 1, -1, 0, 1e-30, 5, -5]
    x[:8] = [1, -1, 0, 0, 0, -1, 1e-30, -1e-30]
    a, _ = oracle.atan2_acos(y, x)
    ref = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    ref[4] = 0.0  # atan2(0, 0) is defined as 0 here
    assert np.abs(a - ref).max() < 1e-6
    c = np.linspace(-1, 1, 20001).astype(np.float32)
    _, ac = oracle.atan2_acos(np.zeros_like(c), c)
    assert np.abs(ac - np.arccos(c.astype(np.float64))).max() < 2e-6


def _dist1d_numpy(data, u):
    """Distribution1D::init / sample (lights.h:28-56) in float32."""
    data = data.astype(np.float32)
    s = np.float32(0)
    for v in data:
        s = np.float32(s + v)
    scale = np.float32(1) / s if s > 0 else np.float32(0)
    pdf = (data * scale).astype(np.float32)
    cdf = np.zeros(data.size + 1, np.float32)
    for i in range(1, data.size):
        cdf[i] = np.float32(cdf[i - 1] + pdf[i - 1])
    cdf[-1] = 1.0
    xs, ps = [], []
    for uu in u:
        idx = int(np.searchsorted(cdf[:data.size], uu, side="right")) - 1
        idx = min(max(idx, 0), data.size - 1)
        t = np.float32((cdf[idx + 1] - uu) / (cdf[idx + 1] - cdf[idx]))
        xs.append(np.float32((1 - t) * idx + t * (idx + 1)))
        ps.append(pdf[idx])
    return np.array(xs, np.float32), np.array(ps, np.float32)


def test_distribution1d_matches_reference_definition():
    rng = np.random.default_rng(1)
    data = rng.uniform(0, 1, 37).astype(np.float32)
    data[[3, 4, 20]] = 0.0  # empty bins are never chosen
    u = rng.uniform(0, 1, 5000).astype(np.float32)
    x, p = oracle.dist1d(data, u)
    xr, pr = _dist1d_numpy(data, u)
    assert np.allclose(x, xr, atol=1e-5) and np.allclose(p, pr, atol=1e-7)
    assert not np.isin(np.floor(x).astype(int), [3, 4, 20]).any() or np.isin(x, [4.0, 5.0, 21.0]).any()
    # the histogram of the samples follows the data
    hist = np.bincount(np.clip(np.floor(x).astype(int), 0, 36), minlength=37) / u.size
    assert np.abs(hist - data / data.sum()).max() < 0.02


def test_oracle_frame_with_sky():
    sc = scenes.icospheres(n_spheres=6, level=2, box=10.0, width=24, height=16, spp=2, max_bounces=3, n_lights=1,
                           rr_start=-1)
    rd = dict(sc.render, rng_mode=0)
    n = rd["width"] * rd["height"]
    pool = np.random.default_rng(3).uniform(1e-6, 1, size=(rd["spp"] * rd["max_bounces"], n, 3)).astype(np.float32)
    base = oracle.OracleScene(sc, use_bvh=False).render(sc.camera, rd, pool)
    sc.lights.append({"type": 1, "map": scenes.procedural_sky(32, 16), "scale": 0.5, "diameter": 20.0,
                      "power": -1.0})
    sky = oracle.OracleScene(sc, use_bvh=False).render(sc.camera, rd, pool)
    assert np.isfinite(sky).all()
    assert sky.mean() > base.mean()  # secondary misses now see the sky
