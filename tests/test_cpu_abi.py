"""CPU-only checks of the C ABI library: it builds, loads, exports every
function include/gbpt.h declares, and refuses cleanly without a GPU."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "gbpt.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    from globillum_gb300 import gbpt
    assert declared_functions() == sorted(gbpt.EXPORTS)


def test_library_exports_every_declared_symbol(lib_path):
    lib = C.CDLL(str(lib_path))
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_no_fallback_when_library_missing(tmp_path):
    from globillum_gb300 import gbpt
    with pytest.raises(FileNotFoundError):
        gbpt.load_library(tmp_path / "libgbpt.so")


def test_layout_sizes(lib_path):
    from globillum_gb300 import gbpt
    lib = gbpt.load_library()
    nb, tb = C.c_int(), C.c_int()
    assert lib.gb_layout_sizes(C.byref(nb), C.byref(tb)) == 0
    assert (nb.value, tb.value) == (80, 48)


def test_null_arguments_are_rejected(lib_path):
    from globillum_gb300 import gbpt
    lib = gbpt.load_library()
    assert lib.gb_ctx_create(None, None) == gbpt.GB_ERR_INVALID
    assert lib.gb_render(None, None, None, None, None, 0) == gbpt.GB_ERR_INVALID
    assert lib.gb_trace_closest(None, None, 0, None, None, None, None, 0) == gbpt.GB_ERR_INVALID
    assert lib.gb_last_error(None) == b"null context"
    lib.gb_ctx_destroy(None)
    lib.gb_scene_destroy(None)


def test_context_without_gpu(lib_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from globillum_gb300 import gbpt
    lib = gbpt.load_library()
    h = C.c_void_p()
    assert lib.gb_ctx_create(C.byref(gbpt.CtxDesc(0, None)), C.byref(h)) == gbpt.GB_ERR_UNSUPPORTED


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors have the size and field offsets of the C structs
    (compiled with gcc from include/gbpt.h)."""
    import shutil
    import subprocess
    from globillum_gb300 import gbpt
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    pairs = {"gb_principled_params": gbpt.PrincipledParams, "gb_material": gbpt.Material, "gb_light": gbpt.Light,
             "gb_scene_desc": gbpt.SceneDesc, "gb_scene_info": gbpt.SceneInfo, "gb_camera": gbpt.Camera,
             "gb_render_desc": gbpt.RenderDesc, "gb_batch_item": gbpt.BatchItem, "gb_hit": gbpt.Hit,
             "gb_stats": gbpt.Stats, "gb_tuning": gbpt.Tuning, "gb_ctx_desc": gbpt.CtxDesc,
             "gb_adjoint_item": gbpt.AdjointItem, "gb_build_options": gbpt.BuildOptions,
             "gb_texture": gbpt.Texture, "gb_bvh_stats": gbpt.BvhStats, "gb_fit_item": gbpt.FitItem}
    c_fields = {"gb_batch_item": ["scene", "camera", "desc", "out_rgb"],
                "gb_tuning": ["refill", "slots", "sample_mb", "tri_mode", "graph", "blocks_per_sm", "stack_depth",
                              "block_threads"],
                "gb_render_desc": ["width", "height", "spp", "max_bounces", "rng_mode", "seed", "ray_offset",
                                   "shadow_offset", "background", "rr_start"],
                "gb_scene_info": ["build_ms", "device_bytes", "overall_light_power", "builder", "build_passes"],
                "gb_stats": ["camera_rays", "kernel_launches", "render_ms", "stage_ms", "stage_launches",
                             "paths_done"]}
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{ROOT / "include" / "gbpt.h"}"',
             "int main(void) {"]
    for name in pairs:
        lines.append(f'  printf("{name} %zu\\n", sizeof({name}));')
    for name, fields in c_fields.items():
        for f in fields:
            lines.append(f'  printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                   check=True).stdout.splitlines())
    for name, cls in pairs.items():
        assert int(got[name]) == C.sizeof(cls), name
    for name, fields in c_fields.items():
        for f in fields:
            assert int(got[f"{name}.{f}"]) == getattr(pairs[name], f).offset, f"{name}.{f}"
