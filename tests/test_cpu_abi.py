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
