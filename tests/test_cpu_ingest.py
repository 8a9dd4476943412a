"""Scene ingest (gb_asset_*, gb_read_pbrdf) on the host: OBJ polygons fanned
into triangles with per-corner or face normals, MTL colours, .pbrdf
principled parameters, the fallback material, transforms, and the
rectangular-light forms of scene scripts.  Fixtures: tests/golden/assets
(written for these tests); the reference's bundled OBJ assets are loaded
too when its tree is available."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from globillum_gb300 import gbpt

ROOT = Path(__file__).resolve().parent.parent

ASSETS = Path(__file__).resolve().parent / "golden" / "assets"


def test_pbrdf_values_and_defaults(tmp_path, lib_path):
    p = gbpt.read_pbrdf(ASSETS / "materials" / "shiny.pbrdf")
    assert p["color"] == pytest.approx((0.2, 0.35, 0.8))
    assert (p["roughness"], p["metallic"], p["specular"]) == pytest.approx((0.25, 0.6, 0.5))
    assert (p["specular_tint"], p["clearcoat"], p["clearcoat_gloss"]) == pytest.approx((0.1, 0.3, 0.7))
    assert (p["opacity"], p["transmiss"], p["anisotropic"]) == (1.0, 1.0, 0.0)  # absent keys: defaults
    f = tmp_path / "glued.pbrdf"
    f.write_text("color 1 1 1\nroughness 0.3\ntransmission0.0\n")  # key glued to its value is skipped
    g = gbpt.read_pbrdf(f)
    assert g["transmiss"] == 1.0 and g["roughness"] == pytest.approx(0.3)
    with pytest.raises(gbpt.GBError):
        gbpt.read_pbrdf(tmp_path / "missing.pbrdf")


def test_obj_room(lib_path):
    a = gbpt.Asset()
    a.add_obj(ASSETS / "room.obj", ASSETS / "materials")
    sd = a.scene_data()
    assert sd.num_triangles == 2 + 2 + 10
    assert a.material_names() == ["gi/fallback", "matte", "shiny"]
    mats = sd.materials
    assert mats[0] == {"diffuse": (1.0, 0.0, 0.0), "principled": -1}
    assert mats[1]["principled"] == -1 and mats[1]["diffuse"] == pytest.approx((0.6, 0.5, 0.4))
    assert mats[2]["principled"] == 0 and sd.params[0]["metallic"] == pytest.approx(0.6)
    # floor: one quad fanned (v1 v2 v3), (v1 v3 v4); no vn -> face normal
    assert np.allclose(sd.positions[0], [0, 0, 0, 4, 0, 0, 4, 0, 4])
    assert np.allclose(sd.positions[1], [0, 0, 0, 4, 0, 4, 0, 0, 4])
    assert np.allclose(sd.normals[0], [0, -1, 0] * 3)
    # wall: negative indices and per-corner normals
    assert np.allclose(sd.positions[2], [0, 0, 4, 4, 0, 4, 4, 3, 4.5])
    assert np.allclose(sd.normals[2], [0, 0.164399, -0.986394] * 3, atol=1e-6)
    assert list(sd.material_index[:4]) == [1, 1, 2, 2]
    assert sd.material_index[4] == 0 and sd.material_index[5] == 0  # unknown material -> fallback
    assert set(sd.material_index[6:]) == {1}
    a.close()


def test_obj_transform(lib_path):
    # mirror in x, scale 2, translate: normals follow the inverse transpose
    M = np.array([[-2, 0, 0, 1], [0, 2, 0, 0], [0, 0, 2, 3], [0, 0, 0, 1]], np.float32)
    a = gbpt.Asset()
    a.add_obj(ASSETS / "room.obj", None, M)
    sd = a.scene_data()
    assert np.allclose(sd.positions[0], [1, 0, 3, -7, 0, 3, -7, 0, 11])
    n = sd.normals[2][:3]
    ref = np.array([0, 0.164399, -0.986394])
    assert np.allclose(n, ref / np.linalg.norm(ref), atol=1e-5)
    # without a material directory every material stays Lambert
    assert all(m["principled"] == -1 for m in sd.materials)
    a.close()


def test_light_script(lib_path):
    a = gbpt.Asset()
    a.add_obj(ASSETS / "room.obj", ASSETS / "materials")
    skipped = a.add_lights(ASSETS / "room.lights.scm")
    assert skipped == 1  # the sky form
    L = a.scene_data().lights
    assert len(L) == 2
    assert L[0]["col"] == (30.0, 25.0, 20.0) and L[0]["center"] == pytest.approx((2.0, 2.9, 2.0))
    assert L[0]["wh"] == pytest.approx((0.8, 0.5)) and L[0]["power"] == -1.0  # add-rectlight's rule
    assert L[1]["dir"] == pytest.approx((0.3, -1.0, 0.2))
    a.close()


def test_ingest_errors(tmp_path, lib_path):
    a = gbpt.Asset()
    with pytest.raises(gbpt.GBError, match="cannot open"):
        a.add_obj(tmp_path / "none.obj")
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nf 1 2 7\n")
    with pytest.raises(gbpt.GBError, match="out of range"):
        a.add_obj(bad)
    s = tmp_path / "bad.scm"
    s.write_text('(light "x" :type :rect :color (list 1 2) :pos (list 0 0 0) :dir (list 0 -1 0) '
                 ':up (list 0 0 1) :dim (list 1 1))')
    with pytest.raises(gbpt.GBError, match="color"):
        a.add_lights(s)
    u = tmp_path / "unbalanced.scm"
    u.write_text('(light "x" :type :rect')
    with pytest.raises(gbpt.GBError, match="malformed"):
        a.add_lights(u)
    a.close()


def _reference_tree():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gbpt_build_ref", ROOT / "oracle" / "build_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.reference_tree()


REF = _reference_tree()


@pytest.mark.skipif(REF is None or not (REF / "boxes.obj").exists(), reason="reference tree not available")
def test_reference_bundled_assets(lib_path):
    """The reference's own OBJ assets and material files load; every face
    of them is a triangle, so the triangle counts equal the face counts."""
    for name in ("boxes.obj", "plainSphere.obj", "bobble-tree.obj"):
        faces = sum(1 for line in (REF / name).open() if line.startswith("f "))
        a = gbpt.Asset()
        a.add_obj(REF / name, REF / "materials")
        sd = a.scene_data()
        assert sd.num_triangles == faces, name
        assert np.isfinite(sd.positions).all() and np.isfinite(sd.normals).all()
        a.close()
    for f in sorted((REF / "materials").glob("*.pbrdf")):
        p = gbpt.read_pbrdf(f)
        assert all(np.isfinite(v) if isinstance(v, float) else np.isfinite(v).all() for v in p.values())
    a = gbpt.Asset()
    a.add_obj(REF / "boxes.obj")
    for script in ("dino.lights.scm", "lights.scm"):
        a.add_lights(REF / script)
    assert len(a.scene_data().lights) >= 1
    a.close()


def test_obj_texture_coordinates_and_ppm_maps(tmp_path, lib_path):
    """vt / "v/vt/vn" corners and MTL map_Kd with PPM images (P6 and P3);
    a map in another format leaves the material untextured."""
    rgb = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3) * 10
    (tmp_path / "tex").mkdir()
    with open(tmp_path / "tex" / "a.ppm", "wb") as f:
        f.write(b"P6\n# comment\n3 2\n255\n" + rgb.tobytes())
    (tmp_path / "b.ppm").write_text("P3\n1 1\n15\n15 0 5\n")
    (tmp_path / "m.mtl").write_text("newmtl A\nKd 1 1 1\nmap_Kd tex/a.ppm\n"
                                    "newmtl B\nKd 0.5 0.5 0.5\nmap_Kd -s 1 1 1 b.ppm\n"
                                    "newmtl C\nKd 0.2 0.2 0.2\nmap_Kd c.png\n")
    (tmp_path / "t.obj").write_text(
        "mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0.25 0.75\nvn 0 0 1\n"
        "usemtl A\nf 1/1/1 2/2/1 3/3/1 4/4/1\nusemtl B\nf 1/1 3/3 4\nusemtl C\nf 1 2 3\n")
    a = gbpt.Asset()
    a.add_obj(tmp_path / "t.obj")
    sd = a.scene_data()
    assert [m["diffuse_texture"] for m in sd.materials] == [-1, 0, 1, -1]
    assert np.array_equal(sd.textures[0][..., :3], rgb) and (sd.textures[0][..., 3] == 255).all()
    assert sd.textures[1][0, 0].tolist() == [255, 0, 85, 255]  # maxval 15 rescaled
    assert np.allclose(sd.texcoords[0], [0, 0, 1, 0, 1, 1]) and np.allclose(sd.texcoords[1], [0, 0, 1, 1, 0.25, 0.75])
    assert np.allclose(sd.texcoords[2], [0, 0, 1, 1, 0, 0])  # the corner without vt
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nf 1/1 2/2 3/1\n")
    with pytest.raises(gbpt.GBError, match="texture coordinate index"):
        a.add_obj(bad)
    a.close()
