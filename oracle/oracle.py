"""ctypes wrapper of the CPU oracle (oracle/gbpt_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from globillum_gb300 import build as _build  # noqa: E402
from globillum_gb300 import gbpt as _gbpt  # noqa: E402

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        lib = C.CDLL(str(path))
        vp, ip, fp = C.c_void_p, C.c_int, C.c_float
        lib.orc_scene_create.restype = vp
        lib.orc_scene_create.argtypes = [ip, vp, vp, vp, ip, vp, ip, vp, ip, vp, ip]
        lib.orc_scene_set_textures.argtypes = [vp, ip, vp, vp, vp]
        lib.orc_scene_destroy.argtypes = [vp]
        lib.orc_scene_destroy.restype = None
        lib.orc_trace_closest.argtypes = [vp, ip, vp, vp, vp, vp, vp]
        lib.orc_trace_any.argtypes = [vp, ip, vp, vp, vp, vp]
        lib.orc_generate_arealight_sample.argtypes = [vp, ip, ip, fp, vp, vp, vp, vp, vp, vp, ip]
        lib.orc_compute_path_contribution_and_bounce.argtypes = [vp, ip, ip, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                                                 vp, vp, ip, ip, ip]
        lib.orc_render.argtypes = [vp, vp, vp, ip, ip, vp, ip, vp, ip, vp]
        lib.orc_adjoint_f64.argtypes = [vp, vp, vp, ip, ip, vp, ip, vp, ip, vp, vp, ip]
        lib.orc_render_direct.argtypes = [vp, vp, vp, ip, vp, ip, vp]
        lib.orc_render_hybrid_direct.argtypes = [vp, vp, vp, ip, ip, vp, ip, vp]
        lib.orc_halton_pool.argtypes = [ip, vp]
        lib.orc_material_sample_eval.argtypes = [vp] * 12
        lib.orc_sincos_2pi.argtypes = [ip, vp, vp, vp]
        lib.orc_shade_eval.argtypes = [vp] * 7
        lib.orc_mrg_jump.argtypes = [C.c_ulonglong, vp, vp]
        lib.orc_atan2_acos.argtypes = [ip, vp, vp, vp, vp]
        lib.orc_dist1d.argtypes = [ip, vp, ip, vp, vp, vp]
        lib.orc64_scene_create.restype = vp
        lib.orc64_scene_create.argtypes = [vp]
        lib.orc64_scene_destroy.argtypes = [vp]
        lib.orc64_scene_destroy.restype = None
        lib.orc64_render.argtypes = [vp, vp, vp, ip, ip, ip, C.c_ulonglong, vp, vp]
        lib.orc64_trace_closest.argtypes = [vp, ip, vp, vp, vp, vp, vp]
        lib.orc_threads.restype = ip
        lib.orc_set_threads.argtypes = [ip]
        lib.orc_set_threads.restype = None
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleScene:
    def __init__(self, scene, use_bvh: bool = True):
        self.lib = load()
        desc, self._keep = _gbpt.make_scene_desc(scene)
        self.h = self.lib.orc_scene_create(desc.num_triangles, desc.positions, desc.normals, desc.material_index,
                                           desc.num_materials, C.cast(desc.materials, C.c_void_p),
                                           desc.num_params, C.cast(desc.params, C.c_void_p), desc.num_lights,
                                           C.cast(desc.lights, C.c_void_p), 1 if use_bvh else 0)
        if not self.h:
            raise ValueError("oracle scene creation failed")
        if desc.diffuse_texture:
            if self.lib.orc_scene_set_textures(self.h, desc.num_textures, C.cast(desc.textures, C.c_void_p),
                                               desc.texcoords, desc.diffuse_texture) != 0:
                raise ValueError("oracle texture set-up failed")

    def close(self):
        if self.h:
            self.lib.orc_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace_closest(self, o, d, tmax, counts: bool = False):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        tmax = np.ascontiguousarray(tmax, np.float32)
        hits = np.empty(tmax.shape[0], _gbpt.HIT_DTYPE)
        c = np.zeros(2, np.uint64)
        self.lib.orc_trace_closest(self.h, tmax.shape[0], _p(o), _p(d), _p(tmax), _p(hits), _p(c))
        return (hits, c) if counts else hits

    def trace_any(self, o, d, tmax):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        tmax = np.ascontiguousarray(tmax, np.float32)
        occ = np.empty(tmax.shape[0], np.uint8)
        self.lib.orc_trace_any(self.h, tmax.shape[0], _p(o), _p(d), _p(tmax), _p(occ))
        return occ

    def render(self, cam: dict, rdesc: dict, pool: np.ndarray, row0: int = 0, row1: int | None = None,
               serial_nee: bool = False, with_stats: bool = False):
        """Progressive frame over rows [row0, row1); pool: (updates, pixels of the rows, 3)."""
        rd = _gbpt.make_render_desc(rdesc)
        cm = _gbpt.make_camera(cam)
        row1 = rd.height if row1 is None else row1
        pool = np.ascontiguousarray(pool, np.float32)
        n = (row1 - row0) * rd.width
        assert pool.shape[1] == n and pool.shape[2] == 3
        out = np.empty((row1 - row0, rd.width, 3), np.float32)
        st = np.zeros(5, np.uint64)
        rc = self.lib.orc_render(self.h, C.byref(cm), C.byref(rd), row0, row1, _p(pool), pool.shape[0], _p(out),
                                 1 if serial_nee else 0, _p(st))
        if rc != 0:
            raise ValueError(f"orc_render failed ({rc})")
        return (out, st) if with_stats else out

    def adjoint_f64(self, cam: dict, rdesc: dict, pool: np.ndarray, dimg: np.ndarray, sel, row0: int = 0,
                    row1: int | None = None, sampling_terms: bool = False) -> np.ndarray:
        """FP64 reference gradient of sum(dimg * image[rows]) with respect to
        the parameters `sel` (gb_scene_param_count layout); sampling_terms
        adds the derivatives of the sampling decisions, as
        gb_ctx_set_gradient_terms(ctx, 1) does."""
        rd = _gbpt.make_render_desc(rdesc)
        cm = _gbpt.make_camera(cam)
        row1 = rd.height if row1 is None else row1
        pool = np.ascontiguousarray(pool, np.float32)
        n = (row1 - row0) * rd.width
        assert pool.shape[1] == n and pool.shape[2] == 3
        g = np.ascontiguousarray(dimg, np.float32).reshape(n, 3)
        sel = np.ascontiguousarray(sel, np.int32)
        out = np.zeros(sel.shape[0], np.float64)
        rc = self.lib.orc_adjoint_f64(self.h, C.byref(cm), C.byref(rd), row0, row1, _p(pool), pool.shape[0], _p(g),
                                      sel.shape[0], _p(sel), _p(out), 1 if sampling_terms else 0)
        if rc != 0:
            raise ValueError(f"orc_adjoint_f64 failed ({rc})")
        return out

    def render_direct(self, cam: dict, rdesc: dict, samples: int, pool: np.ndarray) -> np.ndarray:
        """gpu_area_lights frame; pool: (updates, pixels, 3), updates >= max(1, samples - 1)."""
        rd = _gbpt.make_render_desc(rdesc)
        cm = _gbpt.make_camera(cam)
        pool = np.ascontiguousarray(pool, np.float32)
        out = np.empty((rd.height, rd.width, 3), np.float32)
        rc = self.lib.orc_render_direct(self.h, C.byref(cm), C.byref(rd), int(samples), _p(pool), pool.shape[0],
                                        _p(out))
        if rc != 0:
            raise ValueError(f"orc_render_direct failed ({rc})")
        return out

    def render_hybrid_direct(self, cam: dict, rdesc: dict, cam_samples: int, light_samples: int,
                             pool: np.ndarray) -> np.ndarray:
        """hybrid_area_lights frame; pool: (updates, pixels, 3), updates >= max(C, C * L)."""
        rd = _gbpt.make_render_desc(rdesc)
        cm = _gbpt.make_camera(cam)
        pool = np.ascontiguousarray(pool, np.float32)
        out = np.empty((rd.height, rd.width, 3), np.float32)
        rc = self.lib.orc_render_hybrid_direct(self.h, C.byref(cm), C.byref(rd), int(cam_samples), int(light_samples),
                                               _p(pool), pool.shape[0], _p(out))
        if rc != 0:
            raise ValueError(f"orc_render_hybrid_direct failed ({rc})")
        return out

    def generate_arealight_sample(self, w, h, shadow_offset, rnd, hits, ray_dir, serial=False):
        n = w * h
        ro = np.empty((n, 3), np.float32)
        rd = np.ascontiguousarray(ray_dir, np.float32).copy()
        mt = np.empty(n, np.float32)
        psc = np.empty((n, 3), np.float32)
        self.lib.orc_generate_arealight_sample(self.h, w, h, float(shadow_offset), _p(np.ascontiguousarray(rnd, np.float32)),
                                               _p(hits), _p(ro), _p(rd), _p(mt), _p(psc), 1 if serial else 0)
        return ro, rd, mt, psc

    def compute_path_contribution_and_bounce(self, w, h, rdesc, ray_orig, ray_dir, max_t, hits, occl, rnd, tp,
                                             accum, to_light, psc, path, bounce):
        ro = np.ascontiguousarray(ray_orig, np.float32).copy()
        rd = np.ascontiguousarray(ray_dir, np.float32).copy()
        mt = np.ascontiguousarray(max_t, np.float32).copy()
        t = np.ascontiguousarray(tp, np.float32).copy()
        a = np.ascontiguousarray(accum, np.float32).copy()
        desc = _gbpt.make_render_desc(rdesc)
        self.lib.orc_compute_path_contribution_and_bounce(
            self.h, w, h, C.byref(desc), _p(ro), _p(rd), _p(mt), _p(hits), _p(np.ascontiguousarray(occl, np.uint8)),
            _p(np.ascontiguousarray(rnd, np.float32)), _p(t), _p(a), _p(np.ascontiguousarray(to_light, np.float32)),
            _p(np.ascontiguousarray(psc, np.float32)), path, bounce, 0)
        return ro, rd, mt, t, a


class F64Scene:
    """The independent double-precision restatement (oracle/fp64_render.cpp):
    its own BVH, its own random numbers, every formula re-derived in double.
    Renders converged reference images; rect lights, untextured materials."""

    def __init__(self, scene):
        self.lib = load()
        desc, self._keep = _gbpt.make_scene_desc(scene)
        self.h = self.lib.orc64_scene_create(C.byref(desc))
        if not self.h:
            raise ValueError("fp64 scene creation failed (sky light, texture or bad description)")

    def close(self):
        if self.h:
            self.lib.orc64_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, cam: dict, rdesc: dict, spp: int, seed: int = 1, row0: int = 0, row1: int | None = None,
               with_var: bool = False):
        """Mean radiance (rows, w, 3) float64 over `spp` path samples of rows
        [row0, row1); with_var also returns each pixel's one-sample variance."""
        rd = _gbpt.make_render_desc(rdesc)
        cm = _gbpt.make_camera(cam)
        row1 = rd.height if row1 is None else row1
        mean = np.empty((row1 - row0, rd.width, 3), np.float64)
        var = np.empty_like(mean) if with_var else None
        rc = self.lib.orc64_render(self.h, C.byref(cm), C.byref(rd), row0, row1, int(spp), int(seed), _p(mean),
                                   _p(var))
        if rc != 0:
            raise ValueError(f"orc64_render failed ({rc})")
        return (mean, var) if with_var else mean

    def trace_closest(self, o, d, tmax):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        tmax = np.ascontiguousarray(tmax, np.float32)
        ids = np.empty(tmax.shape[0], np.int32)
        t = np.empty(tmax.shape[0], np.float64)
        self.lib.orc64_trace_closest(self.h, tmax.shape[0], _p(o), _p(d), _p(tmax), _p(ids), _p(t))
        return ids, t


def halton_pool(n: int) -> np.ndarray:
    out = np.empty((n, 2), np.float32)
    load().orc_halton_pool(n, _p(out))
    return out


def sincos_2pi(u: np.ndarray):
    u = np.ascontiguousarray(u, np.float32)
    s = np.empty_like(u)
    c = np.empty_like(u)
    load().orc_sincos_2pi(u.shape[0], _p(u), _p(s), _p(c))
    return s, c


def material_sample_eval(material: dict, params: dict | None, wo_ts, rnd, N, wo_world, wi_eval):
    lib = load()
    m = _gbpt.Material(_gbpt._f3(material["diffuse"]), 0 if params is not None else -1)
    pp = (_gbpt.PrincipledParams * 1)()
    if params is not None:
        sd, _ = _gbpt.make_scene_desc(type("S", (), {
            "positions": np.zeros((1, 9), np.float32), "normals": None, "material_index": np.zeros(1, np.int32),
            "materials": [material], "params": [params], "lights": []})())
        pp[0] = sd.params[0]
    f = lambda v: np.ascontiguousarray(v, np.float32)
    wi = np.empty(3, np.float32)
    pdf = np.empty(1, np.float32)
    lobe = np.empty(1, np.int32)
    fs = np.empty(3, np.float32)
    fe = np.empty(3, np.float32)
    args = [f(wo_ts), f(rnd), f(N), f(wo_world), f(wi_eval)]
    lib.orc_material_sample_eval(C.byref(m), C.cast(pp, C.c_void_p), *[_p(a) for a in args], _p(wi), _p(pdf),
                                 _p(lobe), _p(fs), _p(fe))
    return wi, float(pdf[0]), int(lobe[0]), fs, fe


def shade_eval(diffuse, principled: bool, params18, n_raw, ray_dir, rnd, to_light) -> np.ndarray:
    """sample_bsdf + evaluations (same outputs as the reference glue's ref_shade_eval)."""
    lib = load()
    m = _gbpt.Material(_gbpt._f3(diffuse), 0 if principled else -1)
    pp = _gbpt.PrincipledParams(*[float(x) for x in params18[:12]], _gbpt._f3(params18[12:15]),
                                _gbpt._f3(params18[15:18]))
    f = lambda v: np.ascontiguousarray(v, np.float32)
    out = np.zeros(11, np.float32)
    lib.orc_shade_eval(C.byref(m), C.byref(pp), _p(f(n_raw)), _p(f(ray_dir)), _p(f(rnd)), _p(f(to_light)), _p(out))
    return out


def mrg_jump(steps: int, s1, s2):
    """Library jump-ahead of an MRG32k3a state by `steps` generator steps."""
    a = np.ascontiguousarray(s1, np.uint32).copy()
    b = np.ascontiguousarray(s2, np.uint32).copy()
    load().orc_mrg_jump(int(steps), _p(a), _p(b))
    return a, b


def atan2_acos(y, x):
    """The shared atan2_ex(y, x) and acos_ex(x)."""
    y = np.ascontiguousarray(y, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    a = np.empty_like(x)
    c = np.empty_like(x)
    load().orc_atan2_acos(x.shape[0], _p(y), _p(x), _p(a), _p(c))
    return a, c


def dist1d(data, u):
    """Distribution1D init on `data` and samples at `u`: (x, pdf)."""
    d = np.ascontiguousarray(data, np.float32)
    u = np.ascontiguousarray(u, np.float32)
    x = np.empty_like(u)
    p = np.empty_like(u)
    load().orc_dist1d(d.shape[0], _p(d), u.shape[0], _p(u), _p(x), _p(p))
    return x, p


def mipmaps(rgba: np.ndarray):
    """make_mipmaps of an (h, w, 4) uint8 image: (chain of texels (N, 4), max_mm, size)."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w = img.shape[:2]
    cap = 4 * (2 * w * h + 4 * (w + h) + 64)
    out = np.zeros(cap, np.uint8)
    mm, size = C.c_int(), C.c_int()
    lib = load()
    if lib.orc_mipmaps(_p(img), w, h, _p(out), C.c_longlong(cap), C.byref(mm), C.byref(size)) != 0:
        raise ValueError("mip chain larger than the buffer")
    return out[:4 * size.value].reshape(-1, 4), mm.value, size.value


def tex_sample(rgba: np.ndarray, s, t, diff) -> np.ndarray:
    """sample_bilin_lod of the points (s, t) with footprints diff: (n, 3)."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w = img.shape[:2]
    s, t, diff = (np.ascontiguousarray(a, np.float32) for a in (s, t, diff))
    out = np.empty((s.size, 3), np.float32)
    load().orc_tex_sample(_p(img), w, h, s.size, _p(s), _p(t), _p(diff), _p(out))
    return out


def pow22(x) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty_like(x)
    load().orc_pow22(x.size, _p(x), _p(out))
    return out


def threads() -> int:
    return load().orc_threads()


def set_threads(n: int) -> None:
    load().orc_set_threads(n)
