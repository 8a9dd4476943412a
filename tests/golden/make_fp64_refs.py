"""Writes tests/golden/fp64_refs.npz: converged reference images of the
benchmark workloads, rendered by the oracle's independent double-precision
restatement of the hybrid path (oracle/fp64_render.cpp) at thousands of
samples per pixel.  The GPU frames' RMSE is stated against them (bench.py,
tests/test_gpu_scale.py).  Deterministic: the same code and seeds give the
same file.

Entries (every image float32, rows x width x 3, mean radiance per pixel):
  c1    the 1M-triangle icosphere frame (1280x720, 8 bounces, roulette from
        bounce 3), rows 352-367, 8192 spp
  c0    the Cornell room (256x256, 5 bounces, Halton light samples), whole
        frame, 4096 spp
  c2    the largest scene of the 64-scene mixed set (430,090 triangles,
        256x256, 6 bounces, roulette from bounce 3), rows 112-143, 4096 spp
  c3    the 1M-triangle scene in the adjoint configuration (512x512,
        4 bounces), rows 248-263, 4096 spp
plus per entry: <key>_rows (row0, row1), <key>_spp, <key>_var (mean over
the rows' pixels of the one-sample variance, per channel: the noise of an
n-spp frame is var / n), <key>_check (sum of the scene's positions in double,
to detect a changed generator) and <key>_seed.

    python tests/golden/make_fp64_refs.py [--only c0,c1,...]
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "fp64_refs.npz"


def workloads():
    """(key, scene, render desc, rows, spp, seed) of every entry."""
    from globillum_gb300 import scenes
    c1 = scenes.icospheres()
    c0 = scenes.cornell()
    c2 = scenes.mixed_set()[2]
    c3 = scenes.icospheres()
    r3 = dict(c3.render, width=512, height=512, spp=16, max_bounces=4)
    return [
        ("c1", c1, dict(c1.render), (352, 368), 8192, 101),
        ("c0", c0, dict(c0.render), (0, 256), 4096, 100),
        ("c2", c2, dict(c2.render), (112, 144), 4096, 102),
        ("c3", c3, r3, (248, 264), 4096, 103),
    ]


def checksum(sc) -> float:
    return float(np.sum(sc.positions, dtype=np.float64))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    from oracle import oracle
    only = set(filter(None, args.only.split(",")))
    old = dict(np.load(OUT)) if OUT.exists() else {}
    out = dict(old)
    for key, sc, rd, (r0, r1), spp, seed in workloads():
        if only and key not in only:
            continue
        t0 = time.time()
        f = oracle.F64Scene(sc)
        mean, var = f.render(sc.camera, rd, spp, seed=seed, row0=r0, row1=r1, with_var=True)
        f.close()
        out[key] = mean.astype(np.float32)
        out[key + "_rows"] = np.array([r0, r1], np.int32)
        out[key + "_spp"] = np.int32(spp)
        out[key + "_var"] = var.reshape(-1, 3).mean(axis=0)
        out[key + "_check"] = np.float64(checksum(sc))
        out[key + "_seed"] = np.int64(seed)
        print(f"{key}: rows {r0}-{r1} x {rd['width']} at {spp} spp in {time.time() - t0:.1f} s, "
              f"mean {mean.mean():.5f}, noise of one sample {np.sqrt(out[key + '_var'].mean()):.4f}", flush=True)
    np.savez_compressed(OUT, **out)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
