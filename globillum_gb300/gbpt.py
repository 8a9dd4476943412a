"""ctypes binding of libgbpt.so (include/gbpt.h).

This is the Python form of the binding a reference-side maintainer would add
(the C++ form is include/gb_hybrid_pt.h).  It loads the in-tree library and
raises if it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libgbpt.so"

GB_OK, GB_ERR_INVALID, GB_ERR_CUDA, GB_ERR_OOM, GB_ERR_TIMEOUT, GB_ERR_TRAVERSAL, GB_ERR_UNSUPPORTED = range(7)
GB_LIGHT_RECT, GB_LIGHT_SKY = 0, 1
GB_RNG_MRG32K3A_POOL, GB_RNG_HALTON_LIGHT = 0, 1

F3 = C.c_float * 3


class CtxDesc(C.Structure):
    _fields_ = [("device", C.c_int), ("stream", C.c_void_p)]


class PrincipledParams(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("metallic", "subsurface", "specular", "roughness", "specular_tint",
                                          "anisotropic", "sheen", "sheen_tint", "clearcoat", "clearcoat_gloss",
                                          "opacity", "transmiss")] + [("color", F3), ("tangent", F3)]


class Material(C.Structure):
    _fields_ = [("diffuse", F3), ("principled", C.c_int)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int), ("power", C.c_float), ("center", F3), ("dir", F3), ("up", F3), ("col", F3),
                ("wh", C.c_float * 2), ("sky_rgb", C.c_void_p), ("sky_w", C.c_int), ("sky_h", C.c_int),
                ("sky_scale", C.c_float), ("sky_diameter", C.c_float)]


class Texture(C.Structure):
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("rgba", C.c_void_p)]


class SceneDesc(C.Structure):
    _fields_ = [("num_triangles", C.c_int), ("positions", C.c_void_p), ("normals", C.c_void_p),
                ("material_index", C.c_void_p), ("num_materials", C.c_int), ("materials", C.POINTER(Material)),
                ("num_params", C.c_int), ("params", C.POINTER(PrincipledParams)), ("num_lights", C.c_int),
                ("lights", C.POINTER(Light)), ("num_textures", C.c_int), ("textures", C.POINTER(Texture)),
                ("texcoords", C.c_void_p), ("diffuse_texture", C.c_void_p)]


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_int), ("num_nodes", C.c_int), ("depth", C.c_int), ("binary_nodes", C.c_int),
                ("build_ms", C.c_double), ("device_bytes", C.c_size_t), ("overall_light_power", C.c_float),
                ("builder", C.c_int), ("build_passes", C.c_int)]


GB_BVH_HOST_SAH, GB_BVH_DEVICE_PLOC = 0, 1
BUILDERS = {"host": GB_BVH_HOST_SAH, "device": GB_BVH_DEVICE_PLOC}


class BvhStats(C.Structure):
    _fields_ = [("num_nodes", C.c_int), ("depth", C.c_int), ("binary_nodes", C.c_int), ("num_triangles", C.c_int),
                ("build_ms", C.c_double)]


def bvh_build_stats(positions: np.ndarray, wide_collapse: int = 0, prim_cost: float = 0.0, sah_bins: int = 0) -> dict:
    """gb_bvh_build_stats: the host-built tree of `positions` (n, 9), summarised
    (no device needed)."""
    lib = load_library()
    pos = np.ascontiguousarray(positions, np.float32)
    opts = BuildOptions(GB_BVH_HOST_SAH, 0, int(wide_collapse), float(prim_cost), int(sah_bins))
    st = BvhStats()
    rc = lib.gb_bvh_build_stats(_ptr(pos), int(pos.shape[0]), C.byref(opts), C.byref(st))
    if rc != GB_OK:
        raise GBError(rc, "gb_bvh_build_stats failed")
    return {k: getattr(st, k) for k, _ in BvhStats._fields_}


class BuildOptions(C.Structure):
    _fields_ = [("builder", C.c_int), ("ploc_radius", C.c_int), ("wide_collapse", C.c_int), ("prim_cost", C.c_float),
                ("sah_bins", C.c_int)]


class Camera(C.Structure):
    _fields_ = [("pos", F3), ("dir", F3), ("up", F3), ("fovy_deg", C.c_float), ("aperture", C.c_float),
                ("focus_distance", C.c_float), ("eye_to_lens", C.c_float)]


class RenderDesc(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("spp", C.c_int), ("max_bounces", C.c_int),
                ("rng_mode", C.c_int), ("seed", C.c_uint32), ("ray_offset", C.c_float),
                ("shadow_offset", C.c_float), ("background", F3), ("rr_start", C.c_int)]


class Tuning(C.Structure):
    _fields_ = [("refill", C.c_int), ("slots", C.c_int), ("sample_mb", C.c_int), ("tri_mode", C.c_int),
                ("graph", C.c_int), ("blocks_per_sm", C.c_int), ("stack_depth", C.c_int), ("block_threads", C.c_int)]


class BatchItem(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("desc", RenderDesc), ("out_rgb", C.c_void_p)]


class AdjointItem(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("desc", RenderDesc), ("dL_dimg", C.c_void_p),
                ("dL_dparams", C.c_void_p)]


class FitItem(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("desc", RenderDesc), ("target", C.c_void_p),
                ("image", C.c_void_p)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("beta", C.c_float), ("gamma", C.c_float), ("ref", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("camera_rays", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("closest_node_visits", C.c_uint64), ("closest_tri_tests", C.c_uint64),
                ("shadow_node_visits", C.c_uint64), ("shadow_tri_tests", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("render_ms", C.c_double), ("stage_ms", C.c_double * 6),
                ("stage_launches", C.c_uint64 * 6), ("paths_done", C.c_int), ("light_samples", C.c_uint64)]


HIT_DTYPE = np.dtype([("t", "<f4"), ("beta", "<f4"), ("gamma", "<f4"), ("ref", "<u4")])

# exported symbols of include/gbpt.h (checked by the CPU tests)
EXPORTS = [
    "gb_ctx_create", "gb_ctx_destroy", "gb_last_error", "gb_ctx_set_stream", "gb_scene_create", "gb_scene_destroy",
    "gb_scene_get_info", "gb_render", "gb_render_begin", "gb_render_step", "gb_render_paths_done", "gb_render_read",
    "gb_trace_closest", "gb_trace_any", "gb_generate_arealight_sample", "gb_compute_path_contribution_and_bounce",
    "gb_mrg_pool", "gb_mrg_pool_range", "gb_mrg_states", "gb_get_stats", "gb_render_instrumented", "gb_layout_sizes", "gb_ctx_set_stage_timing",
    "gb_render_noalloc", "gb_ctx_set_tuning", "gb_ctx_get_tuning", "gb_set_fault_injection", "gb_render_batch",
    "gb_autotune", "gb_scene_param_count", "gb_scene_get_params", "gb_scene_set_params", "gb_forward",
    "gb_backward", "gb_backward_batch", "gb_asset_create", "gb_asset_destroy", "gb_asset_last_error",
    "gb_asset_add_obj", "gb_asset_add_lights", "gb_asset_add_light", "gb_asset_get_desc", "gb_asset_material_name",
    "gb_read_pbrdf", "gb_render_direct", "gb_scene_create_ex", "gb_scene_refit", "gb_render_hybrid_direct",
    "gb_bvh_build_stats", "gb_fit_prepare", "gb_fit_step", "gb_ctx_set_gradient_terms",
]

_lib = None


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Loads libgbpt.so; raises FileNotFoundError when it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: run globillum_gb300.build.build_lib() first")
    lib = C.CDLL(str(p))
    vp, ip, fp = C.c_void_p, C.c_int, C.POINTER(C.c_float)
    lib.gb_ctx_create.argtypes = [C.POINTER(CtxDesc), C.POINTER(vp)]
    lib.gb_ctx_destroy.argtypes = [vp]
    lib.gb_ctx_destroy.restype = None
    lib.gb_last_error.argtypes = [vp]
    lib.gb_last_error.restype = C.c_char_p
    lib.gb_ctx_set_stream.argtypes = [vp, vp]
    lib.gb_scene_create.argtypes = [vp, C.POINTER(SceneDesc), C.POINTER(vp)]
    lib.gb_scene_create_ex.argtypes = [vp, C.POINTER(SceneDesc), C.POINTER(BuildOptions), C.POINTER(vp)]
    lib.gb_scene_refit.argtypes = [vp, vp, vp]
    lib.gb_bvh_build_stats.argtypes = [vp, ip, vp, vp]
    lib.gb_scene_destroy.argtypes = [vp]
    lib.gb_scene_destroy.restype = None
    lib.gb_scene_get_info.argtypes = [vp, C.POINTER(SceneInfo)]
    lib.gb_render.argtypes = [vp, vp, C.POINTER(Camera), C.POINTER(RenderDesc), vp, ip]
    lib.gb_render_instrumented.argtypes = [vp, vp, C.POINTER(Camera), C.POINTER(RenderDesc), vp, ip]
    lib.gb_render_begin.argtypes = [vp, vp, C.POINTER(Camera), C.POINTER(RenderDesc)]
    lib.gb_render_step.argtypes = [vp, ip]
    lib.gb_render_paths_done.argtypes = [vp, C.POINTER(C.c_int)]
    lib.gb_render_read.argtypes = [vp, vp, ip]
    lib.gb_trace_closest.argtypes = [vp, vp, ip, vp, vp, vp, vp, ip]
    lib.gb_trace_any.argtypes = [vp, vp, ip, vp, vp, vp, vp, ip]
    lib.gb_generate_arealight_sample.argtypes = [vp, vp, ip, ip, C.c_float, vp, vp, vp, vp, vp, vp]
    lib.gb_compute_path_contribution_and_bounce.argtypes = [vp, vp, ip, ip, C.POINTER(RenderDesc), vp, vp, vp, vp,
                                                            vp, vp, vp, vp, vp, vp, ip, ip]
    lib.gb_mrg_pool.argtypes = [vp, ip, C.c_uint32, ip, ip, vp]
    lib.gb_mrg_pool_range.argtypes = [vp, ip, ip, C.c_uint32, ip, ip, vp]
    lib.gb_mrg_states.argtypes = [vp, C.c_uint32, vp, ip, ip, vp]
    lib.gb_get_stats.argtypes = [vp, C.POINTER(Stats)]
    lib.gb_layout_sizes.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.gb_ctx_set_stage_timing.argtypes = [vp, ip]
    lib.gb_ctx_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    lib.gb_set_fault_injection.argtypes = [ip]
    lib.gb_ctx_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    lib.gb_render_noalloc.argtypes = [vp, C.POINTER(Camera), C.POINTER(RenderDesc), vp, vp]
    lib.gb_render_batch.argtypes = [vp, ip, C.POINTER(BatchItem), ip, ip]
    lib.gb_autotune.argtypes = [vp, ip, C.POINTER(BatchItem), ip, ip, C.POINTER(Tuning), C.POINTER(C.c_double)]
    lib.gb_scene_param_count.argtypes = [vp, C.POINTER(C.c_int)]
    lib.gb_scene_get_params.argtypes = [vp, vp]
    lib.gb_scene_set_params.argtypes = [vp, vp]
    lib.gb_forward.argtypes = [vp, vp, C.POINTER(Camera), C.POINTER(RenderDesc), vp, vp, ip]
    lib.gb_backward.argtypes = [vp, vp, C.POINTER(Camera), C.POINTER(RenderDesc), vp, ip, vp]
    lib.gb_backward_batch.argtypes = [vp, ip, C.POINTER(AdjointItem), ip, ip]
    lib.gb_fit_prepare.argtypes = [vp, ip, C.POINTER(FitItem)]
    lib.gb_ctx_set_gradient_terms.argtypes = [vp, ip]
    lib.gb_fit_step.argtypes = [vp, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_double)]
    lib.gb_asset_create.argtypes = [C.POINTER(vp)]
    lib.gb_asset_destroy.argtypes = [vp]
    lib.gb_asset_destroy.restype = None
    lib.gb_asset_last_error.argtypes = [vp]
    lib.gb_asset_last_error.restype = C.c_char_p
    lib.gb_asset_add_obj.argtypes = [vp, C.c_char_p, C.c_char_p, vp]
    lib.gb_asset_add_lights.argtypes = [vp, C.c_char_p, C.POINTER(C.c_int)]
    lib.gb_asset_add_light.argtypes = [vp, C.POINTER(Light)]
    lib.gb_asset_get_desc.argtypes = [vp, C.POINTER(SceneDesc)]
    lib.gb_asset_material_name.argtypes = [vp, ip, C.POINTER(C.c_char_p)]
    lib.gb_read_pbrdf.argtypes = [C.c_char_p, C.POINTER(PrincipledParams)]
    lib.gb_render_direct.argtypes = [vp, vp, C.POINTER(Camera), C.POINTER(RenderDesc), ip, vp, ip]
    lib.gb_render_hybrid_direct.argtypes = [vp, vp, C.POINTER(Camera), C.POINTER(RenderDesc), ip, ip, vp, ip]
    if path is None:
        _lib = lib
    return lib


class GBError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbpt error {code}: {msg}")
        self.code = code


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f3(v) -> F3:
    return F3(*[float(x) for x in v])


def make_camera(cam: dict) -> Camera:
    return Camera(_f3(cam["pos"]), _f3(cam["dir"]), _f3(cam["up"]), float(cam["fovy_deg"]),
                  float(cam.get("aperture", 0.0)), float(cam.get("focus_distance", 970.0)),
                  float(cam.get("eye_to_lens", 5.0)))


def make_render_desc(r: dict) -> RenderDesc:
    return RenderDesc(int(r["width"]), int(r["height"]), int(r["spp"]), int(r["max_bounces"]),
                      int(r.get("rng_mode", GB_RNG_MRG32K3A_POOL)), int(r.get("seed", 0)),
                      float(r.get("ray_offset", 0.3)), float(r.get("shadow_offset", 0.9)),
                      _f3(r.get("background", (1.0, 1.0, 1.0))), int(r.get("rr_start", -1)))


def make_scene_desc(scene) -> tuple[SceneDesc, list]:
    """SceneDesc for a globillum_gb300.scenes.SceneData; returns (desc, keepalive)."""
    pos = np.ascontiguousarray(scene.positions, dtype=np.float32)
    nrm = None if scene.normals is None else np.ascontiguousarray(scene.normals, dtype=np.float32)
    mid = np.ascontiguousarray(scene.material_index, dtype=np.int32)
    mats = (Material * len(scene.materials))()
    for i, m in enumerate(scene.materials):
        mats[i] = Material(_f3(m["diffuse"]), int(m.get("principled", -1)))
    params = (PrincipledParams * max(1, len(scene.params)))()
    for i, p in enumerate(scene.params):
        params[i] = PrincipledParams(*[float(p.get(k, d)) for k, d in (
            ("metallic", 0), ("subsurface", 0), ("specular", 0), ("roughness", 0), ("specular_tint", 0),
            ("anisotropic", 0), ("sheen", 0), ("sheen_tint", 0), ("clearcoat", 0), ("clearcoat_gloss", 0),
            ("opacity", 1), ("transmiss", 1))], _f3(p.get("color", (0, 0, 0))), _f3(p.get("tangent", (0, 0, 0))))
    lights = (Light * max(1, len(scene.lights)))()
    maps = []
    for i, l in enumerate(scene.lights):
        t = int(l.get("type", GB_LIGHT_RECT))
        if t == GB_LIGHT_SKY:
            # sky: {"type": 1, "map": (h, w, 3) float32 radiance, "scale": s, "diameter": d, "power": -1}
            m = None if l.get("map") is None else np.ascontiguousarray(l["map"], np.float32)
            maps.append(m)
            lights[i] = Light(t, float(l.get("power", -1.0)), F3(), F3(), F3(), F3(), (C.c_float * 2)(),
                              _ptr(m), 0 if m is None else int(m.shape[1]), 0 if m is None else int(m.shape[0]),
                              float(l.get("scale", 1.0)), float(l.get("diameter", 1.0)))
        else:
            lights[i] = Light(t, float(l.get("power", -1.0)), _f3(l["center"]), _f3(l["dir"]),
                              _f3(l.get("up", (0, 0, 1))), _f3(l["col"]), (C.c_float * 2)(*[float(x) for x in l["wh"]]))
    # textures: (h, w, 4) uint8 images, texcoords (n, 6), material key "diffuse_texture"
    texs = [np.ascontiguousarray(t, np.uint8) for t in (getattr(scene, "textures", None) or [])]
    tex_arr = (Texture * max(1, len(texs)))()
    for i, t in enumerate(texs):
        if t.ndim != 3 or t.shape[2] != 4:
            raise ValueError("textures must be (h, w, 4) uint8 arrays")
        tex_arr[i] = Texture(int(t.shape[1]), int(t.shape[0]), _ptr(t))
    tc = getattr(scene, "texcoords", None)
    tc = None if tc is None else np.ascontiguousarray(tc, np.float32)
    dt = np.array([int(m.get("diffuse_texture", -1)) for m in scene.materials], np.int32)
    d = SceneDesc(int(pos.shape[0]), _ptr(pos), _ptr(nrm), _ptr(mid), len(scene.materials), mats,
                  len(scene.params), params, len(scene.lights), lights, len(texs), tex_arr, _ptr(tc),
                  _ptr(dt) if (dt >= 0).any() else None)
    return d, [pos, nrm, mid, mats, params, lights, maps, texs, tex_arr, tc, dt]


class Context:
    """One gb_ctx (one device, one stream)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load_library()
        self.h = C.c_void_p()
        rc = self.lib.gb_ctx_create(C.byref(CtxDesc(device, stream)), C.byref(self.h))
        if rc != GB_OK:
            raise GBError(rc, "gb_ctx_create failed")

    def check(self, rc: int):
        if rc != GB_OK:
            raise GBError(rc, self.lib.gb_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.gb_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream: int | None):
        self.check(self.lib.gb_ctx_set_stream(self.h, stream))

    def scene(self, scene_data, builder: str = "host", ploc_radius: int = 0, wide_collapse: int = 0,
              prim_cost: float = 0.0, sah_bins: int = 0) -> "Scene":
        return Scene(self, scene_data, builder=builder, ploc_radius=ploc_radius, wide_collapse=wide_collapse,
                     prim_cost=prim_cost, sah_bins=sah_bins)

    def stats(self) -> dict:
        s = Stats()
        self.check(self.lib.gb_get_stats(self.h, C.byref(s)))
        d = {k: getattr(s, k) for k, _ in Stats._fields_}
        d["stage_ms"] = list(s.stage_ms)
        d["stage_launches"] = list(s.stage_launches)
        return d

    def set_tuning(self, refill: int = 0, slots: int = 0, sample_mb: int = 0, tri_mode: int = 0, graph: int = 0,
                   blocks_per_sm: int = 0, stack_depth: int = 0, block_threads: int = 0):
        t = Tuning(refill, slots, sample_mb, tri_mode, graph, blocks_per_sm, stack_depth, block_threads)
        self.check(self.lib.gb_ctx_set_tuning(self.h, C.byref(t)))

    def get_tuning(self) -> dict:
        t = Tuning()
        self.check(self.lib.gb_ctx_get_tuning(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    @staticmethod
    def _items(jobs: list, outs: list | None):
        items = (BatchItem * max(1, len(jobs)))()
        for i, (sc, cam, rdesc) in enumerate(jobs):
            items[i] = BatchItem(sc.h, make_camera(cam), make_render_desc(rdesc),
                                 None if outs is None else _ptr(outs[i]))
        return items

    def render_batch(self, jobs: list, graph: bool | None = True, outs: list | None = None) -> list:
        """Renders [(Scene, cam dict, render-desc dict), ...] as one frame
        (gb_render_batch); returns one (h, w, 3) image per job.  graph=None
        follows the context's tuning."""
        if outs is None:
            outs = [np.empty((int(r["height"]), int(r["width"]), 3), dtype=np.float32) for _, _, r in jobs]
        g = -1 if graph is None else (1 if graph else 0)
        self.check(self.lib.gb_render_batch(self.h, len(jobs), self._items(jobs, outs), 0, g))
        return outs

    def render_batch_device(self, jobs: list, out_ptrs: list, graph: bool | None = None) -> None:
        """gb_render_batch into device buffers (one pointer per job)."""
        items = self._items(jobs, None)
        for i, p in enumerate(out_ptrs):
            items[i].out_rgb = C.c_void_p(p)
        g = -1 if graph is None else (1 if graph else 0)
        self.check(self.lib.gb_render_batch(self.h, len(jobs), items, 1, g))

    def backward_batch(self, jobs: list, dimgs: list, graph: bool | None = None) -> list:
        """gb_backward_batch over [(Scene, cam, rdesc), ...] with one image
        gradient per job; returns one parameter gradient per job."""
        items = (AdjointItem * max(1, len(jobs)))()
        keep, outs = [], []
        for i, ((sc, cam, rdesc), g) in enumerate(zip(jobs, dimgs)):
            g = np.ascontiguousarray(g, np.float32)
            o = np.empty(sc.param_count(), np.float32)
            keep.append(g)
            outs.append(o)
            items[i] = AdjointItem(sc.h, make_camera(cam), make_render_desc(rdesc), _ptr(g), _ptr(o))
        gflag = -1 if graph is None else (1 if graph else 0)
        self.check(self.lib.gb_backward_batch(self.h, len(jobs), items, 0, gflag))
        return outs

    def fit_prepare(self, jobs: list, target_ptrs: list, image_ptrs: list | None = None) -> None:
        """gb_fit_prepare over [(Scene, cam, rdesc), ...] with one device
        target image (pointer) per job and optional device image outputs."""
        items = (FitItem * max(1, len(jobs)))()
        for i, (sc, cam, rdesc) in enumerate(jobs):
            img = None if image_ptrs is None else image_ptrs[i]
            items[i] = FitItem(sc.h, make_camera(cam), make_render_desc(rdesc), C.c_void_p(target_ptrs[i]),
                               None if img is None else C.c_void_p(img))
        self._fit_n = len(jobs)
        self._fit_counts = [sc.param_count() for sc, _, _ in jobs]
        self.check(self.lib.gb_fit_prepare(self.h, len(jobs), items))

    def fit_step(self, params: list) -> tuple[list, np.ndarray]:
        """gb_fit_step: one graph launch; returns (gradients, losses)."""
        n = self._fit_n
        xs = [np.ascontiguousarray(p, np.float32) for p in params]
        gs = [np.empty(k, np.float32) for k in self._fit_counts]
        xp = (C.c_void_p * n)(*[x.ctypes.data for x in xs])
        gp = (C.c_void_p * n)(*[g.ctypes.data for g in gs])
        loss = np.empty(n, np.float64)
        self.check(self.lib.gb_fit_step(self.h, xp, gp, loss.ctypes.data_as(C.POINTER(C.c_double))))
        return gs, loss

    def autotune(self, jobs: list, proxy_spp: int = 0, repeats: int = 2) -> tuple[dict, float]:
        """gb_autotune over the batch; returns (best tuning, its frame ms)
        and leaves that tuning set."""
        t = Tuning()
        ms = C.c_double()
        self.check(self.lib.gb_autotune(self.h, len(jobs), self._items(jobs, None), proxy_spp, repeats,
                                        C.byref(t), C.byref(ms)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}, ms.value

    def set_gradient_terms(self, sampling: bool):
        """gb_ctx_set_gradient_terms: add the derivatives of the sampling
        decisions to the adjoint (True) or freeze them (False, default)."""
        self.check(self.lib.gb_ctx_set_gradient_terms(self.h, 1 if sampling else 0))

    def set_stage_timing(self, on: bool):
        self.check(self.lib.gb_ctx_set_stage_timing(self.h, 1 if on else 0))

    def mrg_states(self, subsequences, seed: int = 0, method: int = 1) -> np.ndarray:
        """(n, 6) uint32 states of curand_init(seed, subsequence, 0): method 0
        by curand_init, 1 by the library's jump-ahead."""
        sub = np.ascontiguousarray(subsequences, dtype=np.uint32)
        out = np.empty((sub.size, 6), dtype=np.uint32)
        self.check(self.lib.gb_mrg_states(self.h, seed, _ptr(sub), sub.size, method, _ptr(out)))
        return out

    def mrg_pool(self, npix: int, num_updates: int, first_update: int = 0, seed: int = 0,
                 pixel0: int = 0) -> np.ndarray:
        """(num_updates, npix, 3) pool values of pixels pixel0 .. pixel0 + npix - 1."""
        out = np.empty((num_updates, npix, 3), dtype=np.float32)
        self.check(self.lib.gb_mrg_pool_range(self.h, pixel0, npix, seed, first_update, num_updates, _ptr(out)))
        return out


class Scene:
    """A resident gb_scene."""

    def __init__(self, ctx: Context, scene_data, builder: str = "host", ploc_radius: int = 0,
                 wide_collapse: int = 0, prim_cost: float = 0.0, sah_bins: int = 0):
        """builder: "host" (binned SAH on the CPU) or "device" (PLOC on the
        GPU; refittable); wide_collapse 1: SAH-optimal 8-wide grouping (host)."""
        self.ctx = ctx
        self.h = C.c_void_p()
        desc, self._keep = make_scene_desc(scene_data)
        if builder not in BUILDERS:
            raise ValueError(f"builder must be one of {sorted(BUILDERS)}")
        opts = BuildOptions(BUILDERS[builder], int(ploc_radius), int(wide_collapse), float(prim_cost), int(sah_bins))
        ctx.check(ctx.lib.gb_scene_create_ex(ctx.h, C.byref(desc), C.byref(opts), C.byref(self.h)))

    def refit(self, positions: np.ndarray, normals: np.ndarray | None = None) -> None:
        """gb_scene_refit: moved vertices (n, 9), same triangle order."""
        pos = np.ascontiguousarray(positions, np.float32)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
        if pos.size != 9 * self.info()["num_triangles"] or (nrm is not None and nrm.size != pos.size):
            raise ValueError("positions / normals must hold 9 floats per triangle of the scene")
        self.ctx.check(self.ctx.lib.gb_scene_refit(self.h, _ptr(pos), None if nrm is None else _ptr(nrm)))

    def close(self):
        if self.h:
            self.ctx.lib.gb_scene_destroy(self.h)
            self.h = C.c_void_p()

    def info(self) -> dict:
        i = SceneInfo()
        self.ctx.check(self.ctx.lib.gb_scene_get_info(self.h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in SceneInfo._fields_}

    def render(self, cam: dict, rdesc: dict, instrumented: bool = False, out: np.ndarray | None = None) -> np.ndarray:
        rd = make_render_desc(rdesc)
        if out is None:
            out = np.empty((rd.height, rd.width, 3), dtype=np.float32)
        fn = self.ctx.lib.gb_render_instrumented if instrumented else self.ctx.lib.gb_render
        self.ctx.check(fn(self.ctx.h, self.h, C.byref(make_camera(cam)), C.byref(rd), _ptr(out), 0))
        return out

    def render_device(self, cam: dict, rdesc: dict, out_ptr: int) -> None:
        rd = make_render_desc(rdesc)
        self.ctx.check(self.ctx.lib.gb_render(self.ctx.h, self.h, C.byref(make_camera(cam)), C.byref(rd),
                                              C.c_void_p(out_ptr), 1))

    def render_direct(self, cam: dict, rdesc: dict, light_samples: int = 32) -> np.ndarray:
        """gb_render_direct: the gpu_area_lights image (h, w, 3)."""
        rd = make_render_desc(rdesc)
        out = np.empty((rd.height, rd.width, 3), dtype=np.float32)
        self.ctx.check(self.ctx.lib.gb_render_direct(self.ctx.h, self.h, C.byref(make_camera(cam)), C.byref(rd),
                                                     int(light_samples), _ptr(out), 0))
        return out

    def render_hybrid_direct(self, cam: dict, rdesc: dict, camera_samples: int = 2,
                             light_samples: int = 2) -> np.ndarray:
        """gb_render_hybrid_direct: the hybrid_area_lights image (h, w, 3)."""
        rd = make_render_desc(rdesc)
        out = np.empty((rd.height, rd.width, 3), dtype=np.float32)
        self.ctx.check(self.ctx.lib.gb_render_hybrid_direct(self.ctx.h, self.h, C.byref(make_camera(cam)),
                                                            C.byref(rd), int(camera_samples), int(light_samples),
                                                            _ptr(out), 0))
        return out

    # ------------------------------------------------------ differentiation
    def param_count(self) -> int:
        n = C.c_int()
        self.ctx.check(self.ctx.lib.gb_scene_param_count(self.h, C.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        x = np.empty(self.param_count(), np.float32)
        self.ctx.check(self.ctx.lib.gb_scene_get_params(self.h, _ptr(x)))
        return x

    def set_params(self, x) -> None:
        x = np.ascontiguousarray(x, np.float32)
        assert x.shape == (self.param_count(),)
        self.ctx.check(self.ctx.lib.gb_scene_set_params(self.h, _ptr(x)))

    def forward(self, cam: dict, rdesc: dict, eval_params=None) -> np.ndarray:
        """gb_forward: the image, or with eval_params the frozen-sampling
        replay evaluated at eval_params."""
        rd = make_render_desc(rdesc)
        out = np.empty((rd.height, rd.width, 3), dtype=np.float32)
        ev = None if eval_params is None else np.ascontiguousarray(eval_params, np.float32)
        self.ctx.check(self.ctx.lib.gb_forward(self.ctx.h, self.h, C.byref(make_camera(cam)), C.byref(rd), _ptr(ev),
                                               _ptr(out), 0))
        return out

    def backward(self, cam: dict, rdesc: dict, dimg) -> np.ndarray:
        """gb_backward: dLoss/dparams for dLoss/dimage `dimg` (h, w, 3)."""
        rd = make_render_desc(rdesc)
        g = np.ascontiguousarray(dimg, np.float32)
        assert g.shape == (rd.height, rd.width, 3)
        out = np.empty(self.param_count(), np.float32)
        self.ctx.check(self.ctx.lib.gb_backward(self.ctx.h, self.h, C.byref(make_camera(cam)), C.byref(rd), _ptr(g),
                                                0, _ptr(out)))
        return out

    def backward_device(self, cam: dict, rdesc: dict, dimg_ptr: int) -> np.ndarray:
        """gb_backward with dLoss/dimage in device memory (h*w*3 floats)."""
        rd = make_render_desc(rdesc)
        out = np.empty(self.param_count(), np.float32)
        self.ctx.check(self.ctx.lib.gb_backward(self.ctx.h, self.h, C.byref(make_camera(cam)), C.byref(rd),
                                                C.c_void_p(dimg_ptr), 1, _ptr(out)))
        return out

    def trace_closest(self, orig: np.ndarray, dirs: np.ndarray, max_t: np.ndarray) -> np.ndarray:
        o = np.ascontiguousarray(orig, dtype=np.float32)
        d = np.ascontiguousarray(dirs, dtype=np.float32)
        t = np.ascontiguousarray(max_t, dtype=np.float32)
        n = t.shape[0]
        hits = np.empty(n, dtype=HIT_DTYPE)
        self.ctx.check(self.ctx.lib.gb_trace_closest(self.ctx.h, self.h, n, _ptr(o), _ptr(d), _ptr(t), _ptr(hits), 0))
        return hits

    def trace_any(self, orig: np.ndarray, dirs: np.ndarray, max_t: np.ndarray) -> np.ndarray:
        o = np.ascontiguousarray(orig, dtype=np.float32)
        d = np.ascontiguousarray(dirs, dtype=np.float32)
        t = np.ascontiguousarray(max_t, dtype=np.float32)
        n = t.shape[0]
        occ = np.empty(n, dtype=np.uint8)
        self.ctx.check(self.ctx.lib.gb_trace_any(self.ctx.h, self.h, n, _ptr(o), _ptr(d), _ptr(t), _ptr(occ), 0))
        return occ


_PRINCIPLED_FIELDS = ("metallic", "subsurface", "specular", "roughness", "specular_tint", "anisotropic", "sheen",
                      "sheen_tint", "clearcoat", "clearcoat_gloss", "opacity", "transmiss")


def read_pbrdf(path) -> dict:
    """gb_read_pbrdf: one .pbrdf file as a params dict."""
    lib = load_library()
    p = PrincipledParams()
    rc = lib.gb_read_pbrdf(str(path).encode(), C.byref(p))
    if rc != GB_OK:
        raise GBError(rc, f"cannot read {path}")
    d = {k: float(getattr(p, k)) for k in _PRINCIPLED_FIELDS}
    d["color"] = tuple(float(x) for x in p.color)
    d["tangent"] = tuple(float(x) for x in p.tangent)
    return d


class Asset:
    """gb_asset: OBJ/MTL geometry, .pbrdf materials and light scripts
    gathered into one scene description (host only; no GPU needed)."""

    def __init__(self):
        self.lib = load_library()
        self.h = C.c_void_p()
        if self.lib.gb_asset_create(C.byref(self.h)) != GB_OK:
            raise GBError(GB_ERR_OOM, "gb_asset_create failed")

    def _check(self, rc):
        if rc != GB_OK:
            raise GBError(rc, self.lib.gb_asset_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.gb_asset_destroy(self.h)
            self.h = C.c_void_p()

    def add_obj(self, path, material_dir=None, trafo=None):
        t = None if trafo is None else np.ascontiguousarray(trafo, np.float32).reshape(16)
        self._check(self.lib.gb_asset_add_obj(self.h, str(path).encode(),
                                              None if material_dir is None else str(material_dir).encode(), _ptr(t)))

    def add_lights(self, script_path) -> int:
        """Adds the script's rect lights; returns how many other lights it skipped."""
        n = C.c_int()
        self._check(self.lib.gb_asset_add_lights(self.h, str(script_path).encode(), C.byref(n)))
        return n.value

    def material_names(self) -> list:
        d = SceneDesc()
        self._check(self.lib.gb_asset_get_desc(self.h, C.byref(d)))
        out = []
        for i in range(d.num_materials):
            nm = C.c_char_p()
            self._check(self.lib.gb_asset_material_name(self.h, i, C.byref(nm)))
            out.append(nm.value.decode())
        return out

    def scene_data(self, camera: dict | None = None, render: dict | None = None, name: str = "asset"):
        """The gathered scene as a globillum_gb300.scenes.SceneData (copies)."""
        from .scenes import SceneData
        d = SceneDesc()
        self._check(self.lib.gb_asset_get_desc(self.h, C.byref(d)))
        n = d.num_triangles
        fp = C.POINTER(C.c_float)
        pos = np.ctypeslib.as_array(C.cast(d.positions, fp), shape=(n, 9)).copy() if n else np.zeros((0, 9), np.float32)
        nrm = np.ctypeslib.as_array(C.cast(d.normals, fp), shape=(n, 9)).copy() if n else np.zeros((0, 9), np.float32)
        mid = np.ctypeslib.as_array(C.cast(d.material_index, C.POINTER(C.c_int)), shape=(n,)).copy() if n else \
            np.zeros(0, np.int32)
        mats = [{"diffuse": tuple(float(x) for x in d.materials[i].diffuse), "principled": int(d.materials[i].principled)}
                for i in range(d.num_materials)]
        params = []
        for i in range(d.num_params):
            p = d.params[i]
            q = {k: float(getattr(p, k)) for k in _PRINCIPLED_FIELDS}
            q["color"] = tuple(float(x) for x in p.color)
            q["tangent"] = tuple(float(x) for x in p.tangent)
            params.append(q)
        lights = []
        for i in range(d.num_lights):
            l = d.lights[i]
            lights.append({"type": int(l.type), "power": float(l.power), "center": tuple(l.center), "dir": tuple(l.dir),
                           "up": tuple(l.up), "col": tuple(l.col), "wh": tuple(l.wh)})
        textures, tc = [], None
        if d.diffuse_texture:
            dt = np.ctypeslib.as_array(C.cast(d.diffuse_texture, C.POINTER(C.c_int)), shape=(d.num_materials,))
            for i, m in enumerate(mats):
                m["diffuse_texture"] = int(dt[i])
            for k in range(d.num_textures):
                t = d.textures[k]
                textures.append(np.ctypeslib.as_array(C.cast(t.rgba, C.POINTER(C.c_uint8)),
                                                      shape=(t.h, t.w, 4)).copy())
            tc = np.ctypeslib.as_array(C.cast(d.texcoords, fp), shape=(n, 6)).copy()
        return SceneData(pos.astype(np.float32), nrm.astype(np.float32), mid.astype(np.int32), mats, params, lights,
                         dict(camera or {}), dict(render or {}), name=name, textures=textures, texcoords=tc)
