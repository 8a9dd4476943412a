"""The C++ drop-in (gb::hybrid_pt over the C ABI, driven like the
reference's gi front-end: select -> compute -> update while in_progress)
renders the same image as gb_render."""
import subprocess

import numpy as np
import pytest

from globillum_gb300 import build, scenes

pytestmark = pytest.mark.gpu


def test_headless_matches_gb_render(gpu_ctx, tmp_path):
    exe = build.build_headless()
    sc = scenes.cornell(width=48, height=40, spp=3, max_bounces=4)
    scenes.write_scene_bin(sc, tmp_path / "s.bin")
    r = sc.render
    out = tmp_path / "o.pfm"
    cmd = [str(exe), str(tmp_path / "s.bin"), str(out), "-r", f"{r['width']}x{r['height']}", "-s", str(r["spp"]),
           "-l", str(r["max_bounces"]), "--offsets", repr(r["ray_offset"]), repr(r["shadow_offset"]), "--halton"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    img = scenes.read_pfm(out)
    scene = gpu_ctx.scene(sc)
    ref = scene.render(sc.camera, dict(r))
    scene.close()
    # the file is written like save_image: x and y mirrored
    assert np.array_equal(img, ref[::-1, ::-1])


def test_headless_gpu_area_lights(gpu_ctx, tmp_path):
    """--algo gpu_area_lights selects the C++ gpu_area_lights drop-in
    (registered beside hybrid_pt) and renders gb_render_direct's image."""
    exe = build.build_headless()
    sc = scenes.cornell(width=40, height=32)
    scenes.write_scene_bin(sc, tmp_path / "s.bin")
    out = tmp_path / "d.pfm"
    cmd = [str(exe), str(tmp_path / "s.bin"), str(out), "-r", "40x32", "--algo", "gpu_area_lights",
           "--light-samples", "6"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    img = scenes.read_pfm(out)
    scene = gpu_ctx.scene(sc)
    rd = dict(sc.render, width=40, height=32, seed=0, shadow_offset=0.01, background=(1.0, 1.0, 1.0))
    ref = scene.render_direct(sc.camera, rd, 6)
    scene.close()
    assert np.array_equal(img, ref[::-1, ::-1])


def test_headless_hybrid_area_lights(gpu_ctx, tmp_path):
    """--algo hybrid_area_lights: -s camera samples, --light-samples per
    camera sample, the CPU sampler's shadow offset from --offsets."""
    exe = build.build_headless()
    sc = scenes.cornell(width=40, height=32)
    scenes.write_scene_bin(sc, tmp_path / "s.bin")
    out = tmp_path / "h.pfm"
    cmd = [str(exe), str(tmp_path / "s.bin"), str(out), "-r", "40x32", "--algo", "hybrid_area_lights", "-s", "2",
           "--light-samples", "3", "--offsets", "0.0003", "0.0009"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    img = scenes.read_pfm(out)
    scene = gpu_ctx.scene(sc)
    rd = dict(sc.render, width=40, height=32, seed=0, shadow_offset=0.0009, background=(1.0, 1.0, 1.0))
    ref = scene.render_hybrid_direct(sc.camera, rd, 2, 3)
    scene.close()
    assert np.array_equal(img, ref[::-1, ::-1])


def test_headless_textured_scene(gpu_ctx, tmp_path):
    """Scene file version 3 carries textures: the drop-in renders the
    textured frame of gb_render."""
    exe = build.build_headless()
    sc = scenes.with_textures(scenes.cornell(width=40, height=32, spp=2, max_bounces=3), fraction=1.0, scale=2.0)
    scenes.write_scene_bin(sc, tmp_path / "t.bin")
    r = sc.render
    out = tmp_path / "t.pfm"
    cmd = [str(exe), str(tmp_path / "t.bin"), str(out), "-r", f"{r['width']}x{r['height']}", "-s", str(r["spp"]),
           "-l", str(r["max_bounces"]), "--offsets", repr(r["ray_offset"]), repr(r["shadow_offset"]), "--halton"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    scene = gpu_ctx.scene(sc)
    ref = scene.render(sc.camera, dict(r))
    scene.close()
    assert np.array_equal(scenes.read_pfm(out), ref[::-1, ::-1])
