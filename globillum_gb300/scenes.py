"""Seeded synthetic scenes of the path-tracing workloads.

The reference renders OBJ scenes loaded through Guile scripts
(hl-main.cpp:277-354, scenes.scm); its benchmark scenes are not shipped, so
these generators stand in for them with the shapes, sizes and value
distributions the workloads name:

* ``cornell``: closed room [0,1]^3 of 5 wall quads + 2 boxes = 48 triangles,
  7 Lambert materials with albedo ~ U[0.2, 0.8]^3, one 0.25 x 0.25 ceiling
  light of emission (17, 12, 4), 40 degree pinhole camera, 256 x 256, 16 spp,
  5 bounces, Halton light samples, MRG32k3a path samples.
* ``icospheres``: 800 icospheres of 1280 triangles (icosahedron subdivided
  three times), vertices displaced radially by seeded value noise of
  amplitude 0.1 r, radii lognormal(0, 0.5), centres uniform in [0, 100]^3,
  a 10-triangle ground plane; 256 principled materials (base colour
  U[0,1]^3, roughness U[0.05, 1], metallic Bernoulli(0.3)); 4 rectangular
  lights of side 5 with grey emission U[5, 20]; 1280 x 720, 64 spp,
  8 bounces, Russian roulette from bounce 3.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class SceneData:
    positions: np.ndarray          # (n, 9) float32: a, b, c
    normals: np.ndarray | None     # (n, 9) float32
    material_index: np.ndarray     # (n,) int32
    materials: list                # dicts: diffuse (3), principled (index or -1)
    params: list                   # dicts of PrincipledBRDFParameters fields
    lights: list                   # dicts: center, dir, up, col, wh, power (-1 = rule)
    camera: dict = field(default_factory=dict)
    render: dict = field(default_factory=dict)
    name: str = ""
    textures: list = field(default_factory=list)  # (h, w, 4) uint8 images, row 0 at t = 1
    texcoords: np.ndarray | None = None            # (n, 6) float32: ta, tb, tc

    @property
    def num_triangles(self) -> int:
        return int(self.positions.shape[0])


def _quad(p0, p1, p2, p3, n):
    """Two triangles (p0,p1,p2), (p0,p2,p3) with flat normal n."""
    tri = np.array([p0 + p1 + p2, p0 + p2 + p3], dtype=np.float32)
    nrm = np.array([n * 3, n * 3], dtype=np.float32)
    return tri, nrm


def _grid_quads(origin, du, dv, nu, nv, n):
    tris, nrms = [], []
    o, du, dv = np.array(origin, float), np.array(du, float), np.array(dv, float)
    for i in range(nu):
        for j in range(nv):
            p0 = o + du * i / nu + dv * j / nv
            p1 = o + du * (i + 1) / nu + dv * j / nv
            p2 = o + du * (i + 1) / nu + dv * (j + 1) / nv
            p3 = o + du * i / nu + dv * (j + 1) / nv
            t, m = _quad(list(p0), list(p1), list(p2), list(p3), list(n))
            tris.append(t)
            nrms.append(m)
    return np.concatenate(tris), np.concatenate(nrms)


def _box(lo, hi):
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    faces = [
        ([x0, y0, z0], [x1, y0, z0], [x1, y0, z1], [x0, y0, z1], [0, -1, 0]),
        ([x0, y1, z0], [x0, y1, z1], [x1, y1, z1], [x1, y1, z0], [0, 1, 0]),
        ([x0, y0, z0], [x0, y1, z0], [x1, y1, z0], [x1, y0, z0], [0, 0, -1]),
        ([x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1], [0, 0, 1]),
        ([x0, y0, z0], [x0, y0, z1], [x0, y1, z1], [x0, y1, z0], [-1, 0, 0]),
        ([x1, y0, z0], [x1, y1, z0], [x1, y1, z1], [x1, y0, z1], [1, 0, 0]),
    ]
    tris, nrms = [], []
    for p0, p1, p2, p3, n in faces:
        t, m = _quad(p0, p1, p2, p3, n)
        tris.append(t)
        nrms.append(m)
    return np.concatenate(tris), np.concatenate(nrms)


def cornell(width: int = 256, height: int = 256, spp: int = 16, max_bounces: int = 5, seed: int = 0) -> SceneData:
    """The CPU-runnable plain workload: 48-triangle Cornell-style room."""
    parts = [
        _grid_quads([0, 0, 0], [0, 0, 1], [1, 0, 0], 2, 2, [0, 1, 0]),      # floor
        _grid_quads([0, 1, 0], [1, 0, 0], [0, 0, 1], 2, 2, [0, -1, 0]),     # ceiling
        _grid_quads([0, 0, 1], [1, 0, 0], [0, 1, 0], 2, 1, [0, 0, -1]),     # back wall
        _grid_quads([0, 0, 0], [0, 0, 1], [0, 1, 0], 1, 1, [1, 0, 0]),      # left wall
        _grid_quads([1, 0, 0], [0, 1, 0], [0, 0, 1], 1, 1, [-1, 0, 0]),     # right wall
        _box([0.15, 0.0, 0.45], [0.45, 0.3, 0.75]),                        # short box
        _box([0.55, 0.0, 0.20], [0.85, 0.6, 0.50]),                        # tall box
    ]
    pos = np.concatenate([p[0] for p in parts]).reshape(-1, 9)
    nrm = np.concatenate([p[1] for p in parts]).reshape(-1, 9)
    mid = np.concatenate([np.full(p[0].reshape(-1, 9).shape[0], k, np.int32) for k, p in enumerate(parts)])
    rng = np.random.default_rng(seed)
    albedo = rng.uniform(0.2, 0.8, size=(7, 3)).astype(np.float32)
    materials = [{"diffuse": tuple(map(float, a)), "principled": -1} for a in albedo]
    lights = [{"center": (0.5, 0.995, 0.5), "dir": (0.0, -1.0, 0.0), "up": (0.0, 0.0, 1.0),
               "col": (17.0, 12.0, 4.0), "wh": (0.25, 0.25), "power": -1.0}]
    camera = {"pos": (0.5, 0.5, -1.4), "dir": (0.0, 0.0, 1.0), "up": (0.0, 1.0, 0.0), "fovy_deg": 40.0,
              "aperture": 0.0, "focus_distance": 970.0, "eye_to_lens": 5.0}
    render = {"width": width, "height": height, "spp": spp, "max_bounces": max_bounces, "rng_mode": 1, "seed": 0,
              "ray_offset": 0.3e-3, "shadow_offset": 0.9e-3, "background": (1.0, 1.0, 1.0), "rr_start": -1}
    return SceneData(pos.astype(np.float32), nrm.astype(np.float32), mid, materials, [], lights, camera, render,
                     name="cornell-48tri")


def principled_room(width: int = 48, height: int = 48, spp: int = 16, max_bounces: int = 6,
                    rr_start: int = 2) -> SceneData:
    """The Cornell room with one principled material per part, so that every
    lobe of principledMaterial.h is reached: a rough metal floor, a
    sheen/subsurface ceiling, a clearcoated back wall, an anisotropic metal
    left wall, a Lambert right wall, a glass short box (opacity < 1) and a
    near-mirror tall box; Russian roulette from `rr_start`.  The glass box
    floats 0.01 above the floor: rays inside it reach its bottom face, which
    would otherwise be coplanar with the floor, and which of two coplanar
    faces a float triangle test reports first is a matter of rounding."""
    sc = cornell(width=width, height=height, spp=spp, max_bounces=max_bounces)
    pos = sc.positions.copy()
    glass_box = sc.material_index == 5
    pos[glass_box, 1::3] += np.float32(0.01)
    params = [
        {"color": (0.8, 0.6, 0.3), "metallic": 1.0, "roughness": 0.35},
        {"color": (0.7, 0.7, 0.6), "roughness": 0.6, "sheen": 0.8, "sheen_tint": 0.5, "subsurface": 0.5},
        {"color": (0.3, 0.5, 0.7), "roughness": 0.4, "clearcoat": 1.0, "clearcoat_gloss": 0.7, "specular": 0.5,
         "specular_tint": 0.3},
        {"color": (0.6, 0.7, 0.8), "metallic": 1.0, "roughness": 0.5, "anisotropic": 0.7},
        None,
        {"color": (0.9, 0.9, 0.9), "roughness": 0.2, "opacity": 0.5},
        {"color": (0.9, 0.8, 0.7), "metallic": 1.0, "roughness": 0.06},
    ]
    mats, plist = [], []
    for m, p in zip(sc.materials, params):
        if p is None:
            mats.append(dict(m))
        else:
            mats.append({"diffuse": p["color"], "principled": len(plist)})
            plist.append(p)
    render = dict(sc.render, rng_mode=0, rr_start=rr_start)
    return SceneData(pos, sc.normals, sc.material_index, mats, plist, sc.lights, sc.camera, render,
                     name="principled-room-48tri")


# ------------------------------------------------------------- icospheres --

def icosphere(level: int = 3):
    """Unit icosphere: icosahedron with `level` 4:1 subdivisions (20 * 4^level faces)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, float) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int64)


def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint64) * np.uint64(73856093)) ^ (iy.astype(np.uint64) * np.uint64(19349663)) ^ \
        (iz.astype(np.uint64) * np.uint64(83492791)) ^ np.uint64(seed * 2654435761 % (1 << 32))
    h = (h ^ (h >> np.uint64(13))) * np.uint64(0x5bd1e995)
    h = h ^ (h >> np.uint64(15))
    return (h & np.uint64(0xFFFFFF)).astype(np.float64) / float(0xFFFFFF) * 2.0 - 1.0


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded 3D value noise in [-1, 1]: hashed lattice values, smoothstep-trilinear."""
    fl = np.floor(p)
    f = p - fl
    w = f * f * (3.0 - 2.0 * f)
    i = fl.astype(np.int64) + (1 << 20)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                val = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out += val * wx * wy * wz
    return out


def icospheres(n_spheres: int = 800, level: int = 3, width: int = 1280, height: int = 720, spp: int = 64,
               max_bounces: int = 8, n_materials: int = 256, n_lights: int = 4, box: float = 100.0,
               seed_geometry: int = 1, seed_materials: int = 2, seed_lights: int = 3,
               rr_start: int = 3) -> SceneData:
    """The 1M-triangle GPU workload (800 x 1280 + 10 triangles at the defaults)."""
    uv, uf = icosphere(level)
    rng = np.random.default_rng(seed_geometry)
    radii = rng.lognormal(0.0, 0.5, n_spheres)
    centres = rng.uniform(0.0, box, size=(n_spheres, 3))
    mat_of_sphere = np.random.default_rng(seed_materials + 1000).integers(0, n_materials, n_spheres)
    nv, nf = uv.shape[0], uf.shape[0]
    pos = np.empty((n_spheres * nf + 10, 9), np.float32)
    nrm = np.empty_like(pos)
    mid = np.empty(n_spheres * nf + 10, np.int32)
    for s in range(n_spheres):
        r = radii[s]
        disp = 0.1 * r * value_noise(uv * 2.5 + 17.0 * s, seed_geometry)
        v = centres[s] + uv * (r + disp)[:, None]
        a, b, c = v[uf[:, 0]], v[uf[:, 1]], v[uf[:, 2]]
        fn = np.cross(b - a, c - a)
        vn = np.zeros_like(v)
        for k in range(3):
            np.add.at(vn, uf[:, k], fn)
        vn /= np.linalg.norm(vn, axis=1, keepdims=True)
        sl = slice(s * nf, (s + 1) * nf)
        pos[sl] = np.concatenate([a, b, c], axis=1)
        nrm[sl] = np.concatenate([vn[uf[:, 0]], vn[uf[:, 1]], vn[uf[:, 2]]], axis=1)
        mid[sl] = mat_of_sphere[s]
    # ground plane: 5 quads = 10 triangles below every sphere
    g0, g1, gy = -0.5 * box, 1.5 * box, -0.1 * box
    k = n_spheres * nf
    for q in range(5):
        x0 = g0 + (g1 - g0) * q / 5.0
        x1 = g0 + (g1 - g0) * (q + 1) / 5.0
        t, m = _quad([x0, gy, g0], [x0, gy, g1], [x1, gy, g1], [x1, gy, g0], [0.0, 1.0, 0.0])
        pos[k + 2 * q:k + 2 * q + 2] = t.reshape(2, 9)
        nrm[k + 2 * q:k + 2 * q + 2] = m.reshape(2, 9)
    mid[k:] = 0
    mr = np.random.default_rng(seed_materials)
    params, materials = [], []
    for i in range(n_materials):
        col = mr.uniform(0.0, 1.0, 3)
        rough = mr.uniform(0.05, 1.0)
        metal = 1.0 if mr.uniform() < 0.3 else 0.0
        params.append({"color": tuple(map(float, col)), "roughness": float(rough), "metallic": metal})
        materials.append({"diffuse": tuple(map(float, col)), "principled": i})
    lr = np.random.default_rng(seed_lights)
    lights = []
    for _ in range(n_lights):
        e = float(lr.uniform(5.0, 20.0))
        c = (float(lr.uniform(0.2, 0.8) * box), float(lr.uniform(0.9, 1.1) * box), float(lr.uniform(0.2, 0.8) * box))
        lights.append({"center": c, "dir": (0.0, -1.0, 0.0), "up": (0.0, 0.0, 1.0), "col": (e, e, e),
                       "wh": (5.0, 5.0), "power": -1.0})
    eye = np.array([0.5, 0.7, -0.6]) * box
    look = np.array([0.5, 0.3, 0.5]) * box
    d = look - eye
    d /= np.linalg.norm(d)
    camera = {"pos": tuple(map(float, eye)), "dir": tuple(map(float, d)), "up": (0.0, 1.0, 0.0), "fovy_deg": 45.0,
              "aperture": 0.0, "focus_distance": 970.0, "eye_to_lens": 5.0}
    render = {"width": width, "height": height, "spp": spp, "max_bounces": max_bounces, "rng_mode": 0, "seed": 0,
              "ray_offset": 0.01, "shadow_offset": 0.03, "background": (1.0, 1.0, 1.0), "rr_start": rr_start}
    return SceneData(pos, nrm, mid, materials, params, lights, camera, render,
                     name=f"icospheres-{n_spheres}x{nf}+10tri")


def procedural_sky(width: int = 64, height: int = 32, sun=(0.35, 0.2), seed: int = 0) -> np.ndarray:
    """A lat-long sky radiance map (height rows theta 0..pi, width columns
    phi 0..2 pi, float RGB): a blue-to-white gradient over the upper
    hemisphere, a dim ground, a small bright sun at (theta, phi) / pi,
    2 pi = `sun`, and seeded low-amplitude texel noise.  Stands in for the
    HDR maps add-skylight loads."""
    rng = np.random.default_rng(seed)
    th = (np.arange(height) + 0.5) / height * np.pi
    ph = (np.arange(width) + 0.5) / width * 2 * np.pi
    T, Ph = np.meshgrid(th, ph, indexing="ij")
    up = np.clip(np.cos(T), 0.0, 1.0)[..., None]
    sky = up * np.array([0.3, 0.5, 1.0]) + (1 - up) * np.array([0.9, 0.9, 0.95])
    sky = np.where((T < np.pi / 2)[..., None], sky, np.array([0.15, 0.12, 0.1]))
    st, sp = sun[0] * np.pi, sun[1] * 2 * np.pi
    d2 = (T - st) ** 2 + (np.angle(np.exp(1j * (Ph - sp)))) ** 2
    sky = sky + (np.exp(-d2 / (2 * 0.08 ** 2)) * 40.0)[..., None] * np.array([1.0, 0.9, 0.7])
    sky = sky * (1.0 + 0.05 * rng.standard_normal(sky.shape))
    return np.clip(sky, 0.0, None).astype(np.float32)


def checker_texture(size: int = 64, cells: int = 8, seed: int = 0) -> np.ndarray:
    """(size, size, 4) uint8 checkerboard of two seeded colours with value
    noise on top (so that mip levels differ from the base level)."""
    rng = np.random.default_rng(seed)
    c0, c1 = rng.integers(30, 226, size=(2, 3))
    y, x = np.mgrid[0:size, 0:size]
    chk = ((x * cells // size + y * cells // size) % 2)[..., None]
    img = np.where(chk == 1, c1, c0).astype(np.float64)
    img += rng.integers(-25, 26, size=img.shape)
    out = np.empty((size, size, 4), np.uint8)
    out[..., :3] = np.clip(img, 0, 255).astype(np.uint8)
    out[..., 3] = 255
    return out


def with_textures(scene: SceneData, n_textures: int = 2, size: int = 64, fraction: float = 0.5, scale: float = 1.0,
                  seed: int = 0) -> SceneData:
    """A copy of `scene` with diffuse textures: planar texture coordinates
    (s, t) = scale * (x + z, y + 0.5 z) per corner, n_textures checkerboards,
    each material textured with probability `fraction`."""
    rng = np.random.default_rng(seed)
    p = scene.positions.reshape(-1, 3, 3).astype(np.float64)
    tc = np.stack([scale * (p[..., 0] + p[..., 2]), scale * (p[..., 1] + 0.5 * p[..., 2])], axis=-1)
    mats = []
    for m in scene.materials:
        m = dict(m)
        m["diffuse_texture"] = int(rng.integers(0, n_textures)) if rng.uniform() < fraction else -1
        mats.append(m)
    if all(m["diffuse_texture"] < 0 for m in mats):
        mats[0]["diffuse_texture"] = 0
    return SceneData(scene.positions, scene.normals, scene.material_index, mats, scene.params, scene.lights,
                     dict(scene.camera), dict(scene.render), name=scene.name + "+tex",
                     textures=[checker_texture(size, 4 + 4 * k, seed + k) for k in range(n_textures)],
                     texcoords=tc.reshape(-1, 6).astype(np.float32))


def param_vector(scene: SceneData) -> np.ndarray:
    """The scene's differentiable parameters in gb_scene_param_count order:
    per material base colour, roughness, metallic; per light emission."""
    out = []
    for m in scene.materials:
        if m.get("principled", -1) >= 0:
            p = scene.params[m["principled"]]
            out += list(p.get("color", (0.0, 0.0, 0.0))) + [p.get("roughness", 0.0), p.get("metallic", 0.0)]
        else:
            out += list(m["diffuse"]) + [0.0, 0.0]
    for l in scene.lights:
        out += list(l.get("col", (0.0, 0.0, 0.0)))
    return np.array(out, np.float32)


def mixed_set(n_scenes: int = 64, seed: int = 42, tri_range: tuple = (1_000, 500_000),
              resolutions: tuple = (64, 128, 256, 512), spp_choices: tuple = (4, 16, 64), max_bounces: int = 6,
              n_materials: int = 256, rr_start: int = 3) -> list:
    """The mixed-scene batch workload: icosphere soups whose triangle counts
    are log-uniform in `tri_range`, square resolutions, spp and 1-4 lights
    drawn per scene.  Spheres have 1280 triangles (320 below 1280 triangles
    per scene); the box shrinks with the sphere count so that density stays
    that of the 800-sphere scene."""
    rng = np.random.default_rng(seed)
    out = []
    lo, hi = np.log(tri_range[0]), np.log(tri_range[1])
    for i in range(n_scenes):
        tris = int(np.exp(rng.uniform(lo, hi)))
        level, per = (3, 1280) if tris >= 1280 else (2, 320)
        ns = max(1, int(round((tris - 10) / per)))
        res = int(rng.choice(resolutions))
        spp = int(rng.choice(spp_choices))
        nl = int(rng.integers(1, 5))
        box = 100.0 * (ns / 800.0) ** (1.0 / 3.0)
        sc = icospheres(n_spheres=ns, level=level, width=res, height=res, spp=spp, max_bounces=max_bounces,
                        n_materials=n_materials, n_lights=nl, box=box, seed_geometry=1000 + i,
                        seed_materials=2000 + i, seed_lights=3000 + i, rr_start=rr_start)
        sc.render["seed"] = i
        out.append(sc)
    return out


def random_rays(scene: SceneData, n: int, seed: int = 0, spread: float = 0.2):
    """Seeded rays from points around the scene's bounding box towards random
    points inside it (traversal parity tests)."""
    rng = np.random.default_rng(seed)
    p = scene.positions.reshape(-1, 3)
    lo, hi = p.min(0), p.max(0)
    ext = hi - lo
    o = rng.uniform(lo - spread * ext, hi + spread * ext, size=(n, 3))
    tgt = rng.uniform(lo, hi, size=(n, 3))
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def write_scene_bin(scene: SceneData, path) -> None:
    """Binary scene file read by the headless front-end (host/gi_headless.cpp):
    magic "GBSC", int32 version 3, triangles, materials, params, lights, then
    the gb_scene_desc arrays (gb_light with its sky fields; rect lights only)
    and the gb_camera; then the textures (int32 count, per texture int32 w, h
    and RGBA8 pixels) and an int32 flag followed, when 1, by 6 texture
    coordinates per triangle and a texture index per material.  Little endian."""
    import ctypes as C
    from . import gbpt
    desc, keep = gbpt.make_scene_desc(scene)
    pos = np.ascontiguousarray(scene.positions, np.float32)
    nrm = np.ascontiguousarray(scene.normals, np.float32)
    mid = np.ascontiguousarray(scene.material_index, np.int32)
    with open(path, "wb") as f:
        f.write(b"GBSC")
        f.write(np.array([3, pos.shape[0], len(scene.materials), len(scene.params), len(scene.lights)],
                         np.int32).tobytes())
        f.write(pos.tobytes())
        f.write(nrm.tobytes())
        f.write(mid.tobytes())
        f.write(C.string_at(C.addressof(desc.materials.contents), C.sizeof(gbpt.Material) * len(scene.materials)))
        if scene.params:
            f.write(C.string_at(C.addressof(desc.params.contents), C.sizeof(gbpt.PrincipledParams) * len(scene.params)))
        if scene.lights:
            f.write(C.string_at(C.addressof(desc.lights.contents), C.sizeof(gbpt.Light) * len(scene.lights)))
        cam = gbpt.make_camera(scene.camera)
        f.write(C.string_at(C.addressof(cam), C.sizeof(gbpt.Camera)))
        texs = [np.ascontiguousarray(t, np.uint8) for t in (scene.textures or [])]
        f.write(np.int32(len(texs)).tobytes())
        for t in texs:
            f.write(np.array([t.shape[1], t.shape[0]], np.int32).tobytes())
            f.write(t.tobytes())
        dt = np.array([int(m.get("diffuse_texture", -1)) for m in scene.materials], np.int32)
        textured = scene.texcoords is not None and (dt >= 0).any()
        f.write(np.int32(1 if textured else 0).tobytes())
        if textured:
            f.write(np.ascontiguousarray(scene.texcoords, np.float32).tobytes())
            f.write(dt.tobytes())


def read_pfm(path) -> np.ndarray:
    """Float PFM (as written by gi_headless) -> (h, w, 3) array, top row first."""
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4").reshape(h, w, 3)
    return data[::-1].copy()
