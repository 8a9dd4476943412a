"""Pins the oracle's per-ray arithmetic (globillum_gb300/csrc/gbpt_math.h,
which the GPU kernels share) to the reference's own code.

The golden vectors in tests/golden/ come from the reference's sources
compiled in place (oracle/build_ref.py; generator tests/golden/make_golden.py):
its materialBRDF (principledMaterial.h, simpleMaterial.h, material-wrapper.h)
driven through the sample_material / evaluate_material sequence of
hybrid-pt.cpp:330-371, and rta::generate_arealight_sample of
arealight-sampler-cpu.cpp.  The reference evaluates sin/cos through libm and
some intermediate products in double; the library uses its own float
sin/cos(2 pi u) and float arithmetic, so shading agrees to a relative 1e-4 (every case outside it
is shown to be ill-conditioned: one ulp of input covers the difference)
while the area-light sample (only + - * / sqrt) agrees bit for bit.
"""
from pathlib import Path

import numpy as np
import pytest

from globillum_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden"


def _close(a, b, rtol, atol):
    return np.abs(a.astype(np.float64) - b) <= rtol * np.abs(b.astype(np.float64)) + atol


def _shade_ok(mine, ref, rtol):
    ok_dir = _close(mine[..., 0:3], ref[..., 0:3], 0.0, 2e-5).all(axis=-1)
    ok_pdf = _close(mine[..., 3], ref[..., 3], rtol, 1e-7)
    ok_f = _close(mine[..., 4:10], ref[..., 4:10], rtol, 1e-6).all(axis=-1)
    return ok_dir & ok_pdf & ok_f


def _ulp_nudges(args):
    """The case's inputs with one component of the random numbers, the ray
    direction or the raw normal moved by one ulp either way."""
    for which in (5, 4, 3):  # rnd, ray_dir, n_raw
        for k in range(3):
            for toward in (np.float32(2.0), np.float32(-2.0)):
                a = list(args)
                v = np.array(a[which], np.float32, copy=True)
                v[k] = np.nextafter(v[k], toward, dtype=np.float32)
                a[which] = v
                yield a


def test_shade_matches_reference_golden():
    """Relative 1e-4 on the pdf and BRDF values, 2e-5 on directions.  A case
    outside that must be ill-conditioned: some one-ulp change of one input
    component (the reference evaluates sin/cos through libm and some products
    in double, the library in float) moves the library's result to within
    1e-4 of the reference's.  Such cases are logged and must stay rare."""
    from oracle import oracle
    g = np.load(GOLDEN / "shade_cases.npz")
    ref = g["out"]
    n = ref.shape[0]
    case = lambda i: [g["diffuse"][i], bool(g["principled"][i]), g["params"][i], g["n_raw"][i], g["ray_dir"][i],
                      g["rnd"][i], g["to_light"][i]]
    mine = np.stack([oracle.shade_eval(*case(i)) for i in range(n)])
    assert np.array_equal(mine[:, 10], ref[:, 10]), "glass flag"
    ok = _shade_ok(mine, ref, 1e-4)
    explained = []
    for i in np.flatnonzero(~ok):
        near = [a for a in _ulp_nudges(case(i)) if _shade_ok(oracle.shade_eval(*a), ref[i], 1e-4)]
        assert near, f"case {i} (kind {g['kind'][i]}) differs and is not within one ulp of an input"
        explained.append(int(i))
    print(f"shading cases outside 1e-4 that one ulp of input reproduces: {explained}")
    assert len(explained) <= n // 1000
    # every material family is covered
    for k in range(5):
        assert (g["kind"] == k).sum() > 100


def test_nee_matches_reference_golden_bit_exact():
    from oracle import oracle
    g = np.load(GOLDEN / "nee_cases.npz")
    tris = g["tris"]
    n = g["hits"].shape[0]
    sc = scenes.SceneData(positions=tris[:, :9].copy(), normals=tris[:, 9:].copy(),
                          material_index=np.zeros(tris.shape[0], np.int32),
                          materials=[{"diffuse": (0.5, 0.5, 0.5), "principled": -1}], params=[],
                          lights=[{"center": tuple(c), "dir": tuple(d), "up": (0.0, 0.0, 1.0), "col": tuple(col),
                                   "wh": tuple(wh), "power": float(pw)}
                                  for c, d, col, wh, pw in zip(g["light_center"], g["light_dir"], g["light_col"],
                                                               g["light_wh"], g["light_power"])])
    orc = oracle.OracleScene(sc, use_bvh=False)
    hits = np.ascontiguousarray(g["hits"]).view(oracle._gbpt.HIT_DTYPE).reshape(-1)
    ro, rd, mt, psc = orc.generate_arealight_sample(n, 1, 0.9, g["rnd"], hits, g["ray_dir_in"])
    valid = g["hits"].view(np.uint32)[:, 3] != 0xFFFFFFFF
    assert np.array_equal(mt, g["max_t"])
    assert np.array_equal(ro[valid], g["ray_orig"][valid])
    assert np.array_equal(rd[valid], g["ray_dir"][valid])
    assert np.array_equal(psc[valid], g["psc"][valid])
    assert np.array_equal(psc[~valid], np.zeros_like(psc[~valid]))


def test_live_reference_shading_agrees():
    """Same comparison against a freshly built reference library (skipped
    where the reference tree is not present)."""
    import sys
    sys.path.insert(0, str(GOLDEN))
    import make_golden
    lib = make_golden.load_ref_lib()
    if lib is None:
        pytest.skip("reference tree not present")
    si, _ = make_golden.run_reference(lib, limit=300)
    g = np.load(GOLDEN / "shade_cases.npz")
    assert np.array_equal(si["out"][:300], g["out"][:300]), "golden shading vectors are stale"


def test_sincos_2pi_error_bound():
    from oracle import oracle
    u = np.random.default_rng(0).uniform(0.0, 1.0, 200000).astype(np.float32)
    u = np.concatenate([u, np.array([0.0, 0.25, 0.5, 0.75, 1.0, 0.125], np.float32)])
    s, c = oracle.sincos_2pi(u)
    ang = 2.0 * np.pi * u.astype(np.float64)
    assert np.abs(s - np.sin(ang)).max() < 2.5e-7
    assert np.abs(c - np.cos(ang)).max() < 2.5e-7


def test_halton_pool_follows_util_cpp():
    from oracle import oracle
    pool = oracle.halton_pool(1000)

    def halton(index, base):  # util.cpp:22-32 in float32 arithmetic
        result, f, i = np.float32(0), np.float32(1) / np.float32(base), index
        while i > 0:
            result = np.float32(result + np.float32(f * np.float32(i % base)))
            i //= base
            f = np.float32(f / np.float32(base))
        return result

    for i in [0, 1, 2, 7, 100, 999]:
        assert pool[i, 0] == halton(i + 1, 2) and pool[i, 1] == halton(i + 1, 3)
