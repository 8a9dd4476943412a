"""Build recipe of libgbpt.so (sm_103a kernels + host C++) and of the CPU
oracle library used by the tests.

Everything is compiled in-tree: objects go to ``globillum_gb300/_build`` and
the shared library to ``globillum_gb300/lib/libgbpt.so``.  Device code is
compiled for sm_103a only, with ``-fmad=false`` (fused multiply-adds only
where the sources write ``fmaf``); host code with ``-ffp-contract=off``.  The
oracle is built into ``oracle/_build``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libgbpt.so"
HEADLESS = LIBDIR / "gi_headless"
ORACLE_SRC = ROOT / "oracle" / "gbpt_oracle.cpp"
ORACLE_F64_SRC = ROOT / "oracle" / "fp64_render.cpp"
ORACLE_LIB = ROOT / "oracle" / "_build" / "libgbpt_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_include() -> str:
    nv = Path(_nvcc()).resolve()
    inc = nv.parent.parent / "include"
    return str(inc if inc.exists() else Path("/usr/local/cuda/include"))


def _sources():
    headers = list(CSRC.glob("*.h")) + [ROOT / "include" / "gbpt.h"]
    return headers


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    errors = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(" ".join(c) + "\n" + out)
    if errors:
        raise RuntimeError("build failed:\n" + "\n".join(errors))


def build_lib(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Compiles the CUDA kernels and the C ABI into libgbpt.so."""
    BUILD.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    cu = [CSRC / "gbpt_kernels.cu", CSRC / "gbpt_noalloc.cu", CSRC / "gbpt_build.cu"]
    cpp = [CSRC / "gbpt_api.cpp", CSRC / "gbpt_bvh.cpp", CSRC / "gbpt_ingest.cpp"]
    deps = cu + cpp + _sources()
    # the library records the build-time defines it was made with
    # experimental compile options (GBPT_<name> in the environment -> -DGB_<name>)
    knobs = ("TRAV_MIN_BLOCKS", "SMEM_STACK", "PREFETCH", "SPLIT_NEE", "SHADE_MIN_BLOCKS", "STREAM_MIN_BLOCKS",
             "WIDE_STREAM_GRIDS", "SHADOW_SPLIT", "FUSED_RESTART", "TRI_NOALLOC", "NODE_L2_128", "SHADOW_REFILL", "SHADOW_MIN_BLOCKS",
             "REC_EVICT_FIRST", "NODE_FOLD", "SHADE_EVICT_FIRST", "NODE_L2_PERSIST", "HIT_LINE_KEEP", "TREE_WINDOW", "WIDE_GRID_DIV")
    flags = " ".join(f"GB_{k}={os.environ.get('GBPT_' + k, '')}" for k in knobs)
    stamp = LIB.with_suffix(".flags")
    if not stamp.exists() or stamp.read_text() != flags:
        force = True
    if not force and not _stale(LIB, deps):
        return LIB
    nvcc = _nvcc()
    objs, cmds = [], []
    for s in cu:
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        c = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-ffp-contract=off", "-c", str(s), "-o", str(o)]
        # e.g. GBPT_TRAV_MIN_BLOCKS: resident 128-thread blocks per SM the
        # traversal kernels are compiled for (register budget; default 7)
        for k in knobs:
            v = os.environ.get("GBPT_" + k)
            if v:
                c.insert(1, f"-DGB_{k}={int(v)}")
        if verbose_ptxas:
            c.insert(1, "-Xptxas=-v")
        cmds.append(c)
    defines = [f"-DGB_{k}={int(os.environ['GBPT_' + k])}" for k in knobs if os.environ.get("GBPT_" + k)]
    for s in cpp:
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        cmds.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", *defines, "-I" + _cuda_include(),
                     "-c", str(s), "-o", str(o)])
    _run_parallel(cmds)
    tmp = LIB.with_suffix(".so.tmp")
    _run_parallel([[nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]])
    os.replace(tmp, LIB)
    stamp.write_text(flags)
    return LIB


def build_headless(force: bool = False) -> Path:
    """Builds the headless front-end over include/gb_hybrid_pt.h."""
    lib = build_lib()
    src = PKG / "host" / "gi_headless.cpp"
    deps = [src, ROOT / "include" / "gb_hybrid_pt.h", ROOT / "include" / "gbpt.h", lib]
    if not force and not _stale(HEADLESS, deps):
        return HEADLESS
    tmp = HEADLESS.with_suffix(".tmp")
    _run_parallel([["g++", "-O2", "-std=c++17", str(src), "-o", str(tmp), "-L" + str(LIBDIR), "-lgbpt",
                    "-Wl,-rpath,$ORIGIN"]])
    os.replace(tmp, HEADLESS)
    return HEADLESS


def build_oracle(force: bool = False) -> Path:
    """Compiles the CPU oracle (test infrastructure) into oracle/_build: the
    float restatement of the hybrid path and the independent double-precision
    one (fp64_render.cpp)."""
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    deps = [ORACLE_SRC, ORACLE_F64_SRC, CSRC / "gbpt_math.h", CSRC / "gbpt_host.h", ROOT / "include" / "gbpt.h"]
    if not force and not _stale(ORACLE_LIB, deps):
        return ORACLE_LIB
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    _run_parallel([["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                    str(ORACLE_SRC), str(ORACLE_F64_SRC), "-o", str(tmp)]])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    build_lib(force)
    build_headless(force)
    build_oracle(force)
    ref = ROOT / "oracle" / "build_ref.py"
    if ref.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("gbpt_build_ref", ref)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build_ref(force=force)


if __name__ == "__main__":
    build_all(force=True)
    print(LIB)
