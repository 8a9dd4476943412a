"""Compiles the reference's own CPU code for the pinning tests (test
infrastructure only).

Compiled in place from the reference tree (never copied): the header-only
BRDF code (materialBase.h, simpleMaterial.h, principledParameters.h,
principledMaterial.h, material-wrapper.h, material.h), lights.h, util.h and
arealight-sampler-cpu.cpp, against the shim headers in oracle/ref_shim for
the absent rta / libhyb / libcgls libraries, plus oracle/ref_glue.cpp.
Output: oracle/_ref/libgiref.so.  hybrid-pt.cpp itself is not compiled: its
include chain needs the rta tracer / bouncer class hierarchy.

Without the reference tree (e.g. on a machine that only has this repo) this
is a no-op and returns None.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
# The reference tree this recipe compiles from and the CPU tests read assets
# from: GB_REFERENCE_TREE when set, else the build container's mount.  The
# GPU machine has no reference tree; everything here is then a no-op.
REF_TREE = Path(os.environ.get("GB_REFERENCE_TREE") or "/root/reference")
REF_SRC = REF_TREE / "src"
OUT = HERE / "_ref" / "libgiref.so"


def reference_tree() -> Path | None:
    """The reference tree when it is present, else None."""
    return REF_TREE if (REF_SRC / "arealight-sampler-cpu.cpp").exists() else None


def _cuda_include() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = Path(nvcc).resolve().parent.parent / "include"
    return str(inc if inc.exists() else Path("/usr/local/cuda/include"))


def build_ref(force: bool = False) -> Path | None:
    if reference_tree() is None:
        return None
    srcs = [REF_SRC / "arealight-sampler-cpu.cpp", HERE / "ref_glue.cpp"]
    deps = srcs + list((HERE / "ref_shim").rglob("*.h"))
    if not force and OUT.exists() and all(p.stat().st_mtime <= OUT.stat().st_mtime for p in deps):
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-I" + str(HERE / "ref_shim"), "-I" + str(REF_SRC), "-I" + _cuda_include(),
           *map(str, srcs), "-o", str(tmp)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference pinning build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build_ref(force=True))
