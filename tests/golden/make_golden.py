"""Generates the golden vectors of tests/test_cpu_pinning.py from the
reference's own code (oracle/_ref/libgiref.so, compiled in place from the
reference tree by oracle/build_ref.py).  Needs the reference tree; the
committed .npz files let the tests run without it.

  python tests/golden/make_golden.py

shade_cases.npz  inputs and outputs of ref_shade_eval: the reference's
                 sample_material + evaluate_material sequence
                 (hybrid-pt.cpp:330-371) around materialBRDF on seeded
                 Lambert, principled and glass materials.
nee_cases.npz    inputs and outputs of rta::generate_arealight_sample
                 (arealight-sampler-cpu.cpp:144-156) on a seeded triangle
                 soup with 1-4 rectangular lights.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

PARAM_FIELDS = ["metallic", "subsurface", "specular", "roughness", "specular_tint", "anisotropic", "sheen",
                "sheen_tint", "clearcoat", "clearcoat_gloss", "opacity", "transmiss"]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def shade_inputs(n: int, seed: int = 7):
    rng = np.random.default_rng(seed)
    kind = rng.integers(0, 5, n)  # 0 lambert, 1 principled diffuse, 2 metal, 3 mixed, 4 glass
    diffuse = rng.uniform(0.05, 0.95, (n, 3)).astype(np.float32)
    params = np.zeros((n, 18), np.float32)
    params[:, PARAM_FIELDS.index("opacity")] = 1.0
    params[:, PARAM_FIELDS.index("transmiss")] = 1.0
    params[:, 12:15] = rng.uniform(0.0, 1.0, (n, 3))
    params[:, PARAM_FIELDS.index("roughness")] = rng.uniform(0.05, 1.0, n)
    params[:, PARAM_FIELDS.index("specular")] = rng.uniform(0.0, 1.0, n)
    params[:, PARAM_FIELDS.index("specular_tint")] = rng.uniform(0.0, 1.0, n)
    params[:, PARAM_FIELDS.index("sheen")] = rng.uniform(0.0, 1.0, n) * (rng.uniform(size=n) < 0.5)
    params[:, PARAM_FIELDS.index("sheen_tint")] = rng.uniform(0.0, 1.0, n)
    params[:, PARAM_FIELDS.index("subsurface")] = rng.uniform(0.0, 1.0, n) * (rng.uniform(size=n) < 0.5)
    params[:, PARAM_FIELDS.index("clearcoat")] = rng.uniform(0.0, 1.0, n) * (rng.uniform(size=n) < 0.5)
    params[:, PARAM_FIELDS.index("clearcoat_gloss")] = rng.uniform(0.0, 1.0, n)
    params[:, PARAM_FIELDS.index("anisotropic")] = rng.uniform(0.0, 1.0, n) * (rng.uniform(size=n) < 0.5)
    metal = np.where(kind == 2, 1.0, np.where(kind == 3, rng.uniform(0.0, 1.0, n), 0.0))
    params[:, PARAM_FIELDS.index("metallic")] = metal
    params[kind == 4, PARAM_FIELDS.index("opacity")] = rng.uniform(0.0, 0.99, (kind == 4).sum())
    n_raw = rng.normal(size=(n, 3)) * rng.uniform(0.5, 2.0, (n, 1))
    ray_dir = rng.normal(size=(n, 3))
    rnd = rng.uniform(1e-7, 1.0, (n, 3))
    to_light = rng.normal(size=(n, 3))
    principled = (kind != 0).astype(np.int32)
    return dict(kind=kind.astype(np.int32), principled=principled, diffuse=diffuse, params=params,
                n_raw=n_raw.astype(np.float32), ray_dir=ray_dir.astype(np.float32), rnd=rnd.astype(np.float32),
                to_light=to_light.astype(np.float32))


def nee_inputs(n: int, seed: int = 11):
    rng = np.random.default_rng(seed)
    ntri = 64
    a = rng.uniform(-1.0, 1.0, (ntri, 3))
    tris = np.concatenate([a, a + rng.normal(scale=0.3, size=(ntri, 3)), a + rng.normal(scale=0.3, size=(ntri, 3)),
                           rng.normal(size=(ntri, 9))], axis=1).astype(np.float32)  # positions + normals
    nl = 4
    lights = []
    for _ in range(nl):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        lights.append(dict(center=rng.uniform(-2, 2, 3), dir=d, up=np.array([0.0, 0.0, 1.0]),
                           col=rng.uniform(1.0, 20.0, 3), wh=rng.uniform(0.1, 1.0, 2)))
    hits = np.zeros((n, 4), np.float32)
    beta = rng.uniform(0.0, 1.0, n)
    gamma = rng.uniform(0.0, 1.0, n) * (1.0 - beta)
    hits[:, 0] = rng.uniform(0.1, 5.0, n)
    hits[:, 1] = beta
    hits[:, 2] = gamma
    ref = rng.integers(0, ntri, n).astype(np.uint32)
    miss = rng.uniform(size=n) < 0.1
    hits[miss, 0] = np.float32(3.4028235e38)
    hits.view(np.uint32)[:, 3] = np.where(miss, 0xFFFFFFFF, ref)
    rnd = rng.uniform(1e-7, 1.0, (n, 3)).astype(np.float32)
    ray_dir = rng.normal(size=(n, 3)).astype(np.float32)
    return tris, lights, hits, rnd, ray_dir


def light_array(lights):
    from globillum_gb300 import gbpt
    arr = (gbpt.Light * len(lights))()
    for i, l in enumerate(lights):
        col = [float(x) for x in l["col"]]
        wh = [float(x) for x in l["wh"]]
        power = float(np.float32(np.float32(np.float32(wh[0]) * np.float32(wh[1])) *
                                 np.float32(np.float32(col[0]) + np.float32(col[1]) + np.float32(col[2]))) * .333)
        arr[i] = gbpt.Light(0, power, gbpt._f3(l["center"]), gbpt._f3(l["dir"]), gbpt._f3(l["up"]), gbpt._f3(col),
                            (C.c_float * 2)(*wh))
    return arr


def run_reference(lib, n_shade: int = 4000, n_nee: int = 2000, limit: int | None = None):
    si = shade_inputs(n_shade)
    out = np.zeros((n_shade, 11), np.float32)
    for i in range(n_shade if limit is None else min(limit, n_shade)):
        lib.ref_shade_eval(_p(si["diffuse"][i]), int(si["principled"][i]), _p(si["params"][i]), _p(si["n_raw"][i]),
                           _p(si["ray_dir"][i]), _p(si["rnd"][i]), _p(si["to_light"][i]), _p(out[i]))
    si["out"] = out
    tris, lights, hits, rnd, ray_dir = nee_inputs(n_nee)
    L = light_array(lights)
    overall = np.float32(0.0)
    for i in range(len(lights)):
        overall = np.float32(overall + np.float32(L[i].power))
    ro = np.zeros((n_nee, 3), np.float32)
    rd = ray_dir.copy()
    mt = np.zeros(n_nee, np.float32)
    psc = np.zeros((n_nee, 3), np.float32)
    lib.ref_generate_arealight_sample(n_nee, C.cast(L, C.c_void_p), len(lights), C.c_float(float(overall)), _p(tris),
                                      tris.shape[0], _p(hits), _p(rnd), _p(ro), _p(rd), _p(mt), _p(psc))
    nee = dict(tris=tris, hits=hits, rnd=rnd, ray_dir_in=ray_dir, overall=np.float32(overall),
               light_center=np.array([l["center"] for l in lights], np.float32),
               light_dir=np.array([l["dir"] for l in lights], np.float32),
               light_col=np.array([l["col"] for l in lights], np.float32),
               light_wh=np.array([l["wh"] for l in lights], np.float32),
               light_power=np.array([L[i].power for i in range(len(lights))], np.float32),
               ray_orig=ro, ray_dir=rd, max_t=mt, psc=psc)
    return si, nee


def load_ref_lib():
    sys.path.insert(0, str(ROOT / "oracle"))
    import build_ref  # noqa: E402
    path = build_ref.build_ref()
    if path is None:
        return None
    lib = C.CDLL(str(path))
    lib.ref_shade_eval.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 6
    lib.ref_generate_arealight_sample.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_int,
                                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_void_p]
    return lib


def main():
    lib = load_ref_lib()
    if lib is None:
        raise SystemExit("reference tree not found: cannot generate golden vectors")
    si, nee = run_reference(lib)
    np.savez_compressed(HERE / "shade_cases.npz", **si)
    np.savez_compressed(HERE / "nee_cases.npz", **nee)
    print("wrote", HERE / "shade_cases.npz", HERE / "nee_cases.npz")


if __name__ == "__main__":
    main()
