"""Benchmark of the GB300 path-tracing hot path (one JSON line on rank 0).

Workload: the 1M-triangle plain GPU scene (800 displaced icospheres of 1280
triangles + a 10-triangle ground plane, 256 principled materials, 4 rect
lights, 1280x720, 64 spp, 8 bounces, Russian roulette from bounce 3).  A
step is one full progressive frame (all 64 path samples) with the scene
resident in HBM.  Metric: Mpaths/s = pixels * spp / frame time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbpt|reference]

--impl reference times the CPU restatement of the reference's hybrid path
(oracle/, all host threads) on a bounded sample of the same frame.
Multi-GPU: each rank renders its own copy of the frame (replicas; no
collective), value = all ranks' paths / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# DRAM bytes (read + write) k_extend moves per closest-hit ray on the 1M-triangle
# workload with the default slot pool, from an ncu capture of a whole 16-spp
# frame with a warm L2 (profiles/k_extend_dram_traffic_icospheres1m_16spp.txt).
K_EXTEND_DRAM_BYTES_PER_RAY = 1246.3
METRIC = "Mpaths/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbpt", choices=["gbpt", "reference"])
    ap.add_argument("--workload", default="icospheres-1m", choices=["icospheres-1m", "small"])
    ap.add_argument("--spp", type=int, default=0, help="override the workload's spp (profiling runs)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="minimum CPU-baseline sample time")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--refill", type=int, default=0, help="traversal refill threshold (0 = library default)")
    ap.add_argument("--slots", type=int, default=0, help="paths in flight (0 = library default)")
    ap.add_argument("--tri-mode", type=int, default=0, help="traversal triangle policy 1..3 (0 = library default)")
    ap.add_argument("--graph", type=int, default=0, help="1 = host-driven slot-pool loop, 2 = CUDA graph per chunk")
    ap.add_argument("--builder", default="host", choices=["host", "device"],
                    help="BVH builder of the main scene: binned SAH on the host or PLOC on the GPU")
    ap.add_argument("--wide-collapse", type=int, default=0,
                    help="8-wide grouping: 0 = library default (SAH-optimal), 1 = SAH-optimal, 2 = greedy")
    ap.add_argument("--prim-cost", type=float, default=0.0, help="triangle test cost of the SAH grouping (0 = default)")
    ap.add_argument("--sah-bins", type=int, default=0, help="binned-SAH bins per axis of the host builder (0 = 32)")
    ap.add_argument("--batch-scenes", type=int, default=64, help="scenes of the mixed batch leg (0 = skip it)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the path-replay adjoint leg")
    ap.add_argument("--no-c0", dest="c0", action="store_false", help="skip the Cornell (256^2, 16 spp) leg")
    ap.add_argument("--rmse-spp", type=int, default=1, help="0 = skip the RMSE against the fp64 reference images")
    ap.add_argument("--inverse-iters", type=int, default=200, help="Adam iterations of the inverse leg (0 = skip)")
    return ap.parse_args()


def workload(name: str, spp: int = 0):
    from globillum_gb300 import scenes
    if name == "small":
        sc = scenes.icospheres(n_spheres=50, level=3, box=20.0, width=320, height=180, spp=4, max_bounces=8)
    else:
        sc = scenes.icospheres()
    if spp:
        sc.render["spp"] = spp
    return sc


def config_of(sc, extra=None):
    r = sc.render
    cfg = {"workload": sc.name, "triangles": sc.num_triangles, "width": r["width"], "height": r["height"],
           "spp": r["spp"], "max_bounces": r["max_bounces"], "rr_start": r["rr_start"],
           "materials": len(sc.materials), "lights": len(sc.lights), "bvh": "8-wide compressed (80 B nodes)",
           "l2": "flushed between timed steps (256 MB write)"}
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def frame_pools(sc, ctx=None):
    """The per-pixel MRG32k3a pools of the workload's first path sample
    (updates 0 .. L-1 of curand_init(seed, pixel, 0), hybrid-pt.cpp:83-95),
    made by curand on the GPU as the reference makes them
    (util-kernels.cu:305-333), so that a CPU frame renders the same paths as
    the GPU's first sample.  Without a context: seeded uniform pools."""
    r = sc.render
    n = r["width"] * r["height"]
    if ctx is None:
        return np.random.default_rng(11).uniform(1e-7, 1.0, size=(r["max_bounces"], n, 3)).astype(np.float32), \
            "seeded uniform pools"
    return ctx.mrg_pool(n, r["max_bounces"], seed=r["seed"]), "the GPU frame's MRG32k3a pools (path sample 0)"


def cpu_sample(sc, min_seconds: float, max_frames: int = 64, orc=None, pool=None, serial_nee: bool = False):
    """Times the oracle (CPU restatement of the hybrid path, all host threads)
    on whole frames of the workload at 1 spp until `min_seconds` have passed;
    returns (Mpaths/s, seconds, frames, cores, last image).  serial_nee: the
    reference as it is, whose light-sample loop runs on one thread (the
    misspelt `#pragma omp prallel`, arealight-sampler-cpu.cpp:148).  The BVH
    build is excluded."""
    from oracle import oracle
    rd = dict(sc.render, spp=1)
    own = orc is None
    if own:
        orc = oracle.OracleScene(sc, use_bvh=True)
    if pool is None:
        pool = frame_pools(sc)[0]
    n = rd["width"] * rd["height"]
    total, frames, img = 0.0, 0, None
    while frames < max_frames and (total < min_seconds or frames == 0):
        t0 = time.perf_counter()
        img = orc.render(sc.camera, rd, pool, serial_nee=serial_nee)
        total += time.perf_counter() - t0
        frames += 1
    if own:
        orc.close()
    return n * frames / total / 1e6, total, frames, oracle.threads(), img


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import oracle
    sc = workload(args.workload, args.spp)
    orc = oracle.OracleScene(sc, use_bvh=True)
    ctx = None
    try:  # the pools come from curand on the GPU, as in the reference (util-kernels.cu:305-333)
        import torch
        if torch.cuda.is_available():
            from globillum_gb300 import build, gbpt
            if not build.LIB.exists():
                build.build_lib()
            ctx = gbpt.Context(0)
    except Exception:
        ctx = None
    pool, pool_kind = frame_pools(sc, ctx)
    if ctx is not None:
        ctx.close()
    vals = []
    for i in range(args.warmup + args.steps):
        v, dt, frames, cores, _ = cpu_sample(sc, 0.0, max_frames=1, orc=orc, pool=pool)
        if i >= args.warmup:
            vals.append((v, dt))
    ms = float(np.sum([x[1] for x in vals])) * 1e3 / len(vals)
    v = sc.render["width"] * sc.render["height"] * len(vals) / (ms * len(vals) / 1e3) / 1e6
    # the reference as it is: light samples on one thread (arealight-sampler-cpu.cpp:148)
    v_asis, dt_asis, _, _, _ = cpu_sample(sc, 3.0, max_frames=32, orc=orc, pool=pool, serial_nee=True)
    orc.close()
    sample = f"one whole {sc.render['width']}x{sc.render['height']} frame at 1 spp per step (bounded sample of " \
             f"the {sc.render['spp']}-spp frame), {pool_kind}; light-sample loop on all threads"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_of(sc, {"sample": sample}),
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample},
            "reference_as_is": {"value": v_asis, "unit": METRIC, "cores": cores, "seconds": dt_asis,
                                "note": "the light-sample loop on one thread, as the misspelt pragma of "
                                        "arealight-sampler-cpu.cpp:148 leaves it; shading on all threads"},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


FP64_REFS = ROOT / "tests" / "golden" / "fp64_refs.npz"


def fp64_rmse(img, key: str, spp: int) -> dict:
    """RMSE of a frame (numpy, rows x w x 3) over the rows of the converged
    reference image `key` in tests/golden/fp64_refs.npz (the oracle's
    independent double-precision restatement of the hybrid path, thousands of
    spp, written by tests/golden/make_fp64_refs.py), with the RMSE an
    unbiased spp-sample frame would show (the reference's per-pixel variance)
    and the image-mean difference in standard errors."""
    g = np.load(FP64_REFS)
    r0, r1 = (int(v) for v in g[key + "_rows"])
    ref = g[key].astype(np.float64)
    x = np.asarray(img, np.float64)[r0:r1]
    n_ref, var = int(g[key + "_spp"]), float(g[key + "_var"].mean())
    noise = float(np.sqrt(var * (1.0 / spp + 1.0 / n_ref)))
    return {"value": float(np.sqrt(np.mean((x - ref) ** 2))), "noise_predicted": noise,
            "bias_z": float((x.mean() - ref.mean()) / (noise / np.sqrt(x.size))),
            "reference": f"fp64 oracle, {n_ref} spp (rows {r0}-{r1 - 1})", "image_spp": spp}


def c0_leg(ctx, args, torch, flush, with_cpu: bool):
    """The CPU-runnable configuration: the 48-triangle Cornell room, 256x256,
    16 spp, 5 bounces, Halton light samples, MRG32k3a path samples.  GPU
    frame device-timed (L2 flushed), its RMSE against the fp64 reference of
    the whole frame; on the host, the oracle at the same spp on the same
    pools (as the reference and OpenMP-fixed), whose image is compared with
    the GPU's."""
    from globillum_gb300 import scenes
    sc = scenes.cornell()
    r = sc.render
    W, H, spp = r["width"], r["height"], r["spp"]
    scene = ctx.scene(sc)
    out = torch.empty((H, W, 3), device="cuda", dtype=torch.float32)
    stream = torch.cuda.current_stream()
    # the library's autotuner on this frame (whole frames, 3 repeats); the
    # context's tuning is restored afterwards
    saved = ctx.get_tuning()
    tuning, _ = ctx.autotune([(scene, sc.camera, r)], proxy_spp=0, repeats=3)
    for _ in range(max(1, args.warmup)):
        scene.render_device(sc.camera, r, out.data_ptr())
    ts = []
    for _ in range(max(3, args.steps)):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        scene.render_device(sc.camera, r, out.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    img = out.cpu().numpy()
    ctx.set_tuning(**saved)
    ms = float(np.median(ts))
    res = {"workload": {"scene": sc.name, "triangles": sc.num_triangles, "width": W, "height": H, "spp": spp,
                        "max_bounces": r["max_bounces"], "light_samples": "Halton"},
           "value": W * H * spp / ms / 1e3, "unit": METRIC, "ms_per_frame": ms, "tuning": tuning,
           "rmse": fp64_rmse(img, "c0", spp)}
    if with_cpu:
        from oracle import oracle
        orc = oracle.OracleScene(sc, use_bvh=True)
        pool = ctx.mrg_pool(W * H, spp * r["max_bounces"], seed=r["seed"])
        for serial, name in ((False, "cpu_openmp_fixed"), (True, "cpu_reference_as_is")):
            dt, frames = 0.0, 0
            while dt < 2.0 and frames < 32:  # whole frames, at least 2 s of CPU time
                t0 = time.perf_counter()
                cimg = orc.render(sc.camera, r, pool, serial_nee=serial)
                dt += time.perf_counter() - t0
                frames += 1
            res[name] = {"value": W * H * spp * frames / dt / 1e6, "unit": METRIC, "seconds": dt, "frames": frames,
                         "cores": oracle.threads(), "image_equals_gpu": bool(np.array_equal(cimg, img))}
        res["rmse"]["cpu_frame"] = fp64_rmse(cimg, "c0", spp)["value"]
        orc.close()
    scene.close()
    return res


def batch_leg(ctx, args, torch, flush, dist):
    """Mixed-scene batch (64 icosphere soups, log-uniform 1K-500K triangles,
    64^2-512^2 pixels, 4/16/64 spp, 1-4 lights, 6 bounces): knobs picked by
    gb_autotune on the whole batch frame, then the batched frame
    (gb_render_batch) against the plain form (one gb_render per scene, in
    sequence), both device-timed with L2 flushed between steps, and against
    the sum of each scene's best frame time rendered alone.  Images of the
    two forms are bit-identical (checked here), so RMSE is equal."""
    from globillum_gb300 import replicas, scenes
    t0 = time.perf_counter()
    mixed = scenes.mixed_set(args.batch_scenes)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    handles = [ctx.scene(sc) for sc in mixed]
    build_s = time.perf_counter() - t0
    jobs = [(h, sc.camera, sc.render) for h, sc in zip(handles, mixed)]
    paths = sum(sc.render["width"] * sc.render["height"] * sc.render["spp"] for sc in mixed)
    outs = [torch.empty((sc.render["height"], sc.render["width"], 3), device="cuda", dtype=torch.float32)
            for sc in mixed]
    ptrs = [o.data_ptr() for o in outs]
    saved = ctx.get_tuning()
    t0 = time.perf_counter()
    tuning, tune_ms = ctx.autotune(jobs, proxy_spp=0, repeats=3)
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ts = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.sum(ts))

    def plain():
        for (h, cam, rd), p in zip(jobs, ptrs):
            h.render_device(cam, rd, p)

    def batched():
        ctx.render_batch_device(jobs, ptrs)

    plain_ms = timed(plain)
    plain_imgs = [o.clone() for o in outs]

    def best_single():
        """Sum over the scenes of each one's best frame time rendered alone
        (CUDA events around the one call, L2 flushed before it): the plain
        form without the gaps between calls."""
        tot = 0.0
        for (h, cam, rd), p in zip(jobs, ptrs):
            h.render_device(cam, rd, p)
            best = float("inf")
            for _ in range(max(1, args.steps)):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                h.render_device(cam, rd, p)
                e1.record(stream)
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1))
            tot += best
        return tot

    best_single_ms = best_single()
    batch_ms = timed(batched)
    big = int(np.argmax([sc.num_triangles for sc in mixed]))
    rmse_big = (fp64_rmse(outs[big].cpu().numpy(), "c2", mixed[big].render["spp"])
                if big == 2 and args.rmse_spp > 0 else None)
    launches = ctx.stats()["kernel_launches"]
    same = all(torch.equal(a, b) for a, b in zip(plain_imgs, outs))
    tot_b, ms_b = replicas.aggregate(paths * args.steps, batch_ms, dist, "cuda")
    tot_p, ms_p = replicas.aggregate(paths * args.steps, plain_ms, dist, "cuda")
    vb, vp = replicas.mpaths_per_s(tot_b, ms_b), replicas.mpaths_per_s(tot_p, ms_p)
    for h in handles:
        h.close()
    ctx.set_tuning(**saved)
    tris = [sc.num_triangles for sc in mixed]
    return {"value": vb, "unit": METRIC, "plain_value": vp, "batched_over_plain": vb / vp,
            "ms_per_step": ms_b / args.steps, "plain_ms_per_step": ms_p / args.steps,
            "best_single_sum_ms": best_single_ms,
            "batched_over_best_single": best_single_ms / (ms_b / args.steps),
            "images_identical": bool(same), "paths_per_step": paths, "launches_per_step": int(launches),
            "rmse_largest_scene": rmse_big,
            "workload": {"scenes": len(mixed), "triangles_total": int(sum(tris)), "triangles_min": int(min(tris)),
                         "triangles_max": int(max(tris)), "resolutions": [64, 128, 256, 512], "spp": [4, 16, 64],
                         "max_bounces": 6, "generate_s": gen_s, "bvh_build_and_upload_s": build_s},
            "autotune": {"tuning": tuning, "frame_ms": tune_ms, "seconds": tune_s, "proxy_spp": None}}


def adjoint_leg(ctx, scene, sc, args, torch, flush, orc):
    """Path-replay adjoint on the 1M-triangle scene at 512x512, 16 spp, 4
    bounces: L2 loss against a target rendered from the same geometry with
    independently seeded material parameters; gradients for all materials'
    base colour, roughness, metallic and all lights' emission.  Times
    forward (gb_render) and backward (gb_backward) on the device, checks the
    gradient on 32 seeded parameters against central differences (h = 1e-3)
    of gb_forward(eval_params) at common random numbers and, on the CPU,
    against the oracle's FP64 dual-number replay of the same paths."""
    from globillum_gb300 import scenes
    rd = dict(sc.render, width=512, height=512, spp=16, max_bounces=4)
    H, W = rd["height"], rd["width"]
    x0 = scene.get_params()
    tgt_sc = scenes.icospheres(n_spheres=1, seed_materials=97)  # materials only; geometry unused
    xt = x0.copy()
    xt[:5 * len(sc.materials)] = scenes.param_vector(tgt_sc)[:5 * len(sc.materials)]
    scene.set_params(xt)
    target = torch.empty((H, W, 3), device="cuda", dtype=torch.float32)
    scene.render_device(sc.camera, rd, target.data_ptr())
    scene.set_params(x0)
    img = torch.empty_like(target)
    stream = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    fwd_ms = timed(lambda: scene.render_device(sc.camera, rd, img.data_ptr()))
    rmse_fwd = fp64_rmse(img.cpu().numpy(), "c3", rd["spp"]) if args.rmse_spp > 0 else None
    dimg = (2.0 * (img - target)).contiguous()
    grad_box = {}

    def bwd():
        grad_box["g"] = scene.backward_device(sc.camera, rd, dimg.data_ptr())

    bwd_ms = timed(bwd)
    grad = grad_box["g"]
    loss0 = float(((img - target) ** 2).sum().item())
    # finite differences of the frozen-sampling forward, 32 seeded parameters
    rng = np.random.default_rng(2024)
    live = np.flatnonzero(np.abs(grad) > 1e-4 * np.abs(grad).max())
    sel = np.sort(rng.choice(live, size=min(32, live.size), replace=False))
    tgt_np = target.cpu().numpy().astype(np.float64)
    h = 1e-3
    fd = []
    for i in sel:
        xp, xm = x0.copy(), x0.copy()
        xp[i] += h
        xm[i] -= h
        lp = float(((scene.forward(sc.camera, rd, xp).astype(np.float64) - tgt_np) ** 2).sum())
        lm = float(((scene.forward(sc.camera, rd, xm).astype(np.float64) - tgt_np) ** 2).sum())
        fd.append((lp - lm) / (2 * h))
    fd = np.array(fd)
    rel_fd = np.abs(grad[sel] - fd) / np.maximum(np.abs(fd), 1e-12)
    # the frame is only piecewise smooth (per-channel throughput clamp at 1):
    # an outlier is re-checked with a 3x smaller step to show whether a kink
    # lies within +-h
    outliers = []
    for j in np.flatnonzero(rel_fd > 1e-3):
        i = sel[j]
        hs = h / 3.0
        xp, xm = x0.copy(), x0.copy()
        xp[i] += hs
        xm[i] -= hs
        lp = float(((scene.forward(sc.camera, rd, xp).astype(np.float64) - tgt_np) ** 2).sum())
        lm = float(((scene.forward(sc.camera, rd, xm).astype(np.float64) - tgt_np) ** 2).sum())
        f2 = (lp - lm) / (2 * hs)
        outliers.append({"param": int(i), "rel_err_h": float(rel_fd[j]),
                         "rel_err_h/3": float(abs(grad[i] - f2) / max(abs(f2), 1e-12)),
                         "grad_over_max": float(abs(grad[i]) / np.abs(grad).max())})
    out = {"workload": {"scene": sc.name, "width": W, "height": H, "spp": rd["spp"], "max_bounces": rd["max_bounces"],
                        "params": int(x0.size), "loss": "L2 to a target from materials seeded 97"},
           "forward_ms": fwd_ms, "backward_ms": bwd_ms, "backward_over_forward": bwd_ms / fwd_ms, "loss": loss0,
           "tuning": ctx.get_tuning(),
           "rmse_forward_frame": rmse_fwd,
           "adjoint_record_bytes": int(80 * rd["max_bounces"] * min(W * H * rd["spp"], 1 << 22)),
           "finite_differences": {"h": h, "params": int(sel.size), "median_rel_err": float(np.median(rel_fd)),
                                  "max_rel_err": float(rel_fd.max()),
                                  "within_1e-3": int((rel_fd <= 1e-3).sum()), "outliers": outliers,
                                  "chosen_from": "parameters with |grad| > 1e-4 max|grad|, seeded",
                                  "sampling": "frozen at the current parameters (gb_forward eval_params)"}}
    if orc is not None:
        pool = ctx.mrg_pool(W * H, rd["spp"] * rd["max_bounces"], seed=rd["seed"])
        t0 = time.perf_counter()
        ref = orc.adjoint_f64(sc.camera, rd, pool, dimg.cpu().numpy(), sel)
        rel64 = np.abs(grad[sel].astype(np.float64) - ref) / np.maximum(np.abs(ref), 1e-12)
        out["fp64_replay"] = {"params": int(sel.size), "median_rel_err": float(np.median(rel64)),
                              "max_rel_err": float(rel64.max()), "cpu_seconds": time.perf_counter() - t0}
    return out


def inverse_leg(ctx, args, torch, dist):
    """Batched inverse rendering: 16 icosphere scenes (10K-200K triangles,
    256x256, 8 spp, 4 bounces, 64 principled materials, 1-4 lights).  Each
    scene's 64 materials (base colour, roughness, metallic) are recovered
    from a target rendered with hidden seeded parameters: Adam (lr 1e-2) on
    the summed L2 image losses, starting from the scenes' own seeded
    materials, with the knobs gb_autotune picks for this batch.  One
    iteration = one gb_fit_step: a single CUDA graph launch
    that uploads the parameters, renders the batched forward frame, forms
    the losses and image gradients on the device and runs the batched
    adjoint; the host applies the parameter Jacobian and Adam.  The same
    iteration is also timed as 16 sequential plain runs (gb_render +
    gb_backward per scene, image gradients through the host)."""
    from globillum_gb300 import scenes
    n_sc = 16
    mixed = scenes.mixed_set(n_sc, seed=77, tri_range=(10_000, 200_000), resolutions=(256,), spp_choices=(8,),
                             max_bounces=4, n_materials=64)
    handles = [ctx.scene(sc) for sc in mixed]
    jobs = [(h, sc.camera, sc.render) for h, sc in zip(handles, mixed)]
    nmp = 5 * 64
    x_init = [h.get_params() for h in handles]
    x_hidden = []
    for i, (h, x0) in enumerate(zip(handles, x_init)):
        xh = x0.copy()
        xh[:nmp] = scenes.param_vector(scenes.icospheres(n_spheres=1, n_materials=64,
                                                         seed_materials=5000 + i))[:nmp]
        x_hidden.append(xh)
    # targets with the hidden parameters
    targets = []
    for h, xh, (_, cam, rd) in zip(handles, x_hidden, jobs):
        h.set_params(xh)
        targets.append(torch.from_numpy(h.render(cam, rd)).cuda())
    for h, x0 in zip(handles, x_init):
        h.set_params(x0)
    outs = [torch.empty_like(t) for t in targets]
    ptrs = [o.data_ptr() for o in outs]
    # one parameter vector per scene (scenes have 1-4 lights); only the
    # materials are free
    paths = sum(sc.render["width"] * sc.render["height"] * sc.render["spp"] for sc in mixed)

    def param_err(xs, visible=None):
        e = {}
        for name, k in (("colour", [0, 1, 2]), ("roughness", [3]), ("metallic", [4])):
            sq = []
            for i in range(n_sc):
                ms = range(64) if visible is None else np.flatnonzero(visible[i])
                idx = np.array([5 * m + j for m in ms for j in k], dtype=np.int64)
                if idx.size:
                    sq.append((xs[i][idx] - x_hidden[i][idx]) ** 2)
            e[name] = float(np.sqrt(np.mean(np.concatenate(sq)))) if sq else None
        return e

    # knobs for this batch from the library's autotuner (restored at the end)
    saved = ctx.get_tuning()
    tuning, _ = ctx.autotune(jobs, proxy_spp=0, repeats=3)
    # one fitting step = one CUDA graph launch: parameter upload, batched
    # forward frame, L2 loss and image gradient on the device, batched
    # adjoint, gradient reduction (gb_fit_step)
    ctx.fit_prepare(jobs, [t.data_ptr() for t in targets], ptrs)

    def fit(sampling):
        """Adam from the initial materials with the frozen-sampling gradient
        or with the derivatives of the sampling decisions."""
        ctx.set_gradient_terms(sampling)
        xs_t = [torch.tensor(x0, requires_grad=True) for x0 in x_init]
        opt = torch.optim.Adam(xs_t, lr=1e-2)
        visible = None
        losses, t_iter = [], []
        for it in range(args.inverse_iters):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g, lv = ctx.fit_step([x.detach().numpy() for x in xs_t])
            t_iter.append(time.perf_counter() - t0)
            losses.append(float(lv.sum()))
            if visible is None:
                # materials that influence their image: colour-gradient norm
                # at the start above 1 % of the scene's largest
                visible = []
                for gi in g:
                    gn = np.linalg.norm(gi[:nmp].reshape(64, 5)[:, :3], axis=1)
                    visible.append(gn > 1e-2 * max(gn.max(), 1e-30))
            for x, gi in zip(xs_t, g):
                gt = torch.from_numpy(gi)
                gt[nmp:] = 0.0
                x.grad = gt
            opt.step()
            with torch.no_grad():
                for x in xs_t:
                    x[:nmp] = x[:nmp].clamp(0.0, 1.0)
        ctx.set_gradient_terms(False)
        xs = [x.detach().numpy() for x in xs_t]
        return {"gradient": "sampling decisions differentiated" if sampling else "frozen sampling",
                "param_rmse_final": param_err(xs),
                "visible_materials": int(sum(int(v.sum()) for v in visible)) if visible is not None else 0,
                "param_rmse_initial_visible": param_err(x_init, visible) if visible is not None else None,
                "param_rmse_final_visible": param_err(xs, visible) if visible is not None else None,
                "loss_first": losses[0] if losses else None, "loss_last": losses[-1] if losses else None,
                }, t_iter

    err0 = param_err(x_init)
    fits = {}
    t_iter = []
    for name, sampling in (("frozen", False), ("sampling", True)):
        fits[name], t = fit(sampling)
        t_iter += t[1:] if len(t) > 1 else t
    # the same iteration as 16 sequential plain runs (gb_render + gb_backward per scene)
    seq = []
    for _ in range(max(3, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for (h, cam, rd), p, t in zip(jobs, ptrs, targets):
            h.render_device(cam, rd, p)
        for (h, cam, rd), o, t in zip(jobs, outs, targets):
            h.backward(cam, rd, (2.0 * (o - t)).cpu().numpy())
        torch.cuda.synchronize()
        seq.append(time.perf_counter() - t0)
    for h, x0 in zip(handles, x_init):
        h.close()
    ctx.set_tuning(**saved)
    it_s = float(np.median(t_iter))
    seq_s = float(np.median(seq))
    return {"workload": {"scenes": n_sc, "triangles": [int(sc.num_triangles) for sc in mixed], "resolution": 256,
                         "spp": 8, "max_bounces": 4, "materials_per_scene": 64, "iterations": args.inverse_iters,
                         "optimizer": "Adam lr 1e-2 on base colour, roughness, metallic"},
            "param_rmse_initial": err0, "fits": fits, "tuning": tuning,
            "iteration_ms": it_s * 1e3, "sequential_iteration_ms": seq_s * 1e3,
            "batched_over_sequential": seq_s / it_s,
            "mpaths_per_s_fwd_plus_bwd": 2 * paths / it_s / 1e6,
            "graph_launches_per_iteration": 1,
            "note": "wall-clock per iteration: one gb_fit_step (parameter records built on the host, one graph "
                    "launch, parameter Jacobian on the host); Adam on the host"}


def run_gbpt(args, rank, world):
    import torch
    from globillum_gb300 import build, gbpt
    if not build.LIB.exists():  # an existing build is used as it is (with its own compile options)
        build.build_lib()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sc = workload(args.workload, args.spp)
    r = sc.render
    W, H, spp = r["width"], r["height"], r["spp"]
    stream = torch.cuda.current_stream()
    ctx = gbpt.Context(local, stream.cuda_stream)
    if args.refill or args.slots or args.tri_mode or args.graph:
        ctx.set_tuning(refill=args.refill, slots=args.slots, tri_mode=args.tri_mode, graph=args.graph)
    t0 = time.perf_counter()
    scene = ctx.scene(sc, builder=args.builder, wide_collapse=args.wide_collapse, prim_cost=args.prim_cost,
                      sah_bins=args.sah_bins)
    upload_s = time.perf_counter() - t0
    info = scene.info()
    out = torch.empty((H, W, 3), device="cuda", dtype=torch.float32)
    flush = torch.empty(64 * 1024 * 1024, device="cuda", dtype=torch.float32)  # 256 MB > L2

    for _ in range(args.warmup):
        scene.render_device(sc.camera, r, out.data_ptr())
    torch.cuda.synchronize()

    # device-timed steps (scene resident, L2 flushed between steps)
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    times, launches = [], 0
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        scene.render_device(sc.camera, r, out.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        launches += ctx.stats()["kernel_launches"]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()

    # per-stage times of one more frame (CUDA events around every stage
    # launch; the slot-pool loop then runs from the host)
    ctx.set_stage_timing(True)
    flush.zero_()
    scene.render_device(sc.camera, r, out.data_ptr())
    torch.cuda.synchronize()
    st_stage = ctx.stats()
    stage_ms = np.array(st_stage["stage_ms"])
    stage_n = np.array(st_stage["stage_launches"])
    stage_frame_ms = st_stage["render_ms"]
    ctx.set_stage_timing(False)
    from globillum_gb300 import replicas
    paths = W * H * spp
    paths_total, total_ms = replicas.aggregate(paths * args.steps, float(np.sum(times)), dist, "cuda")
    value = replicas.mpaths_per_s(paths_total, total_ms)

    # end to end: through the C ABI with a pinned host image, copies inside
    host = torch.empty((H, W, 3), dtype=torch.float32).pin_memory()
    host_np = host.numpy()
    torch.cuda.synchronize()
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        scene.render(sc.camera, r, out=host_np)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = float(np.sum(e2e_t))
    e2e_val = paths * args.steps * world / e2e_s / 1e6
    import ctypes
    h2d = ctypes.sizeof(gbpt.Camera) + ctypes.sizeof(gbpt.RenderDesc)

    # traversal work of the same frame (instrumented render, outside timing)
    scene.render_device(sc.camera, r, out.data_ptr())
    scene.render(sc.camera, r, instrumented=True)
    ist = ctx.stats()
    node_b, tri_b = 80, 36
    ext_rays = ist["camera_rays"] + ist["extension_rays"]
    trav_bytes = ist["closest_node_visits"] * node_b + ist["closest_tri_tests"] * tri_b + ext_rays * 48
    # the light sample k_extend takes at every hit, and a miss's end of path:
    # per hit the hit triangle's positions and normals (72 B), the light
    # record (64 B), one draw of three uniforms (12 B), the shadow ray out
    # (32 B) and its potential contribution (12 B); per miss the throughput
    # and accumulation in (24 B) and the sample out (12 B)
    hits = ist["light_samples"]
    misses = ext_rays - hits
    closest_bytes = trav_bytes + hits * (72 + 64 + 12 + 32 + 12) + misses * 36
    ext_ms = stage_ms[1]          # per frame
    ext_launches = stage_n[1]
    peak, peak_kind = measured_peaks()
    achieved = closest_bytes / (ext_ms / 1e3) / 1e9 if ext_ms > 0 else None
    achieved_trav = trav_bytes / (ext_ms / 1e3) / 1e9 if ext_ms > 0 else None
    # FP32 work of the traversal: ~24 flops per child slab test (8 children
    # per node visit), ~30 per triangle test
    trav_flops = ist["closest_node_visits"] * 8 * 24 + ist["closest_tri_tests"] * 30
    fp32_tflops = trav_flops / (ext_ms / 1e3) / 1e12 if ext_ms > 0 else None
    rays = ist["camera_rays"] + ist["extension_rays"] + ist["shadow_rays"]
    mrays = rays / (total_ms / args.steps / 1e3) / 1e6

    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_of(sc, {"parallelism": f"replicas x{world}", "bvh_build_ms": info["build_ms"],
                                     "bvh_builder": args.builder, "wide_collapse": args.wide_collapse,
                                     "scene_upload_s": upload_s, "bvh_nodes": info["num_nodes"],
                                     "bvh_depth": info["depth"], "tuning": ctx.get_tuning()}),
            "mrays_per_s": mrays,
            "rays_per_frame": {"camera": ist["camera_rays"], "extension": ist["extension_rays"],
                               "shadow": ist["shadow_rays"]},
            "traversal_per_ray": {"closest_node_visits": ist["closest_node_visits"] / max(1, ext_rays),
                                  "closest_tri_tests": ist["closest_tri_tests"] / max(1, ext_rays),
                                  "shadow_node_visits": ist["shadow_node_visits"] / max(1, ist["shadow_rays"]),
                                  "shadow_tri_tests": ist["shadow_tri_tests"] / max(1, ist["shadow_rays"])},
            "stage_ms_per_frame": {"path_start": stage_ms[0], "closest_hit+light_sample": ext_ms,
                                   "any_hit+restart_of_misses": stage_ms[2], "shade+restart": stage_ms[3],
                                   "iteration_end": stage_ms[4],
                                   "moving_average": stage_ms[5], "frame_ms_with_stage_events": stage_frame_ms},
            "stage_launches_per_frame": [int(x) for x in stage_n],
            "roofline": {"bound": "hbm", "kernel": "k_extend (closest-hit traversal + light sample)",
                         "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None,
                         "traffic": (K_EXTEND_DRAM_BYTES_PER_RAY * ext_rays / max(1.0, ext_launches)
                                     if args.workload == "icospheres-1m" else None),
                         "traffic_source": "ncu dram__bytes_read+write of k_extend per closest-hit ray "
                                           "(warm L2, whole 16-spp frame of this workload) x rays per launch",
                         "algorithmic_bytes_per_launch": closest_bytes / max(1.0, ext_launches),
                         "bytes_model": "per ray: node visits*80 + tri tests*36 + 32 ray in + 16 hit out; per hit "
                                        "(light sample): 72 hit triangle positions+normals + 64 light + 12 draw + "
                                        "32 shadow ray out + 12 potential contribution; per miss: 24 in + 12 "
                                        "sample out (counts from the instrumented render of the same frame)",
                         "traversal_only": {"achieved": achieved_trav,
                                            "frac": (achieved_trav / peak) if achieved_trav else None,
                                            "bytes_per_launch": trav_bytes / max(1.0, ext_launches),
                                            "bytes_model": "node visits*80 + tri tests*36 + 48 per ray"},
                         "closest_hits_per_frame": int(hits), "misses_per_frame": int(misses),
                         "fp32": {"achieved_tflops": fp32_tflops,
                                  "model": "node visits*8*24 + tri tests*30 flops (slab tests of 8 children, "
                                           "Moller-Trumbore), no measured FP32 peak to divide by"}},
            "clocks": clocks,
            "e2e": {"value": e2e_val, "unit": METRIC, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": W * H * 3 * 4},
            "gpu_launches": int(launches)}
    if args.rmse_spp > 0 and args.workload == "icospheres-1m" and spp == 64:
        # the timed frame against the converged fp64 reference of its rows
        # 352-367 (an independent double-precision restatement, its own random
        # numbers); batched and CPU frames are bit-identical to this frame's
        scene.render_device(sc.camera, r, out.data_ptr())
        torch.cuda.synchronize()
        line["rmse"] = fp64_rmse(out.cpu().numpy(), "c1", spp)
    if args.batch_scenes > 0:
        line["batched"] = batch_leg(ctx, args, torch, flush, dist)
    orc = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle
        orc = oracle.OracleScene(sc, use_bvh=True)
    if not args.no_adjoint:
        line["adjoint"] = adjoint_leg(ctx, scene, sc, args, torch, flush, orc)
    if args.inverse_iters > 0:
        line["inverse"] = inverse_leg(ctx, args, torch, dist)
    if args.c0:
        line["c0"] = c0_leg(ctx, args, torch, flush, orc is not None)
    if orc is not None:
        pool, pool_kind = frame_pools(sc, ctx)
        v, dt, frames, cores, cimg = cpu_sample(sc, args.cpu_seconds, orc=orc, pool=pool)
        v1, dt1, _, _, _ = cpu_sample(sc, 3.0, max_frames=32, orc=orc, pool=pool, serial_nee=True)
        scene.render_device(sc.camera, dict(r, spp=1), out.data_ptr())
        same1 = bool(np.array_equal(cimg, out.cpu().numpy()))
        line["cpu_baseline"] = {"value": v, "unit": METRIC, "cores": cores, "kind": "port",
                                "sample": f"{frames} whole {W}x{H} frames at 1 spp ({dt:.1f} s of CPU time, "
                                          f"BVH build excluded), {pool_kind}",
                                "image_equals_gpu_1spp_frame": same1,
                                "reference_as_is": {"value": v1, "unit": METRIC, "seconds": dt1,
                                                    "note": "light-sample loop on one thread "
                                                            "(arealight-sampler-cpu.cpp:148)"}}
        if "rmse" in line:
            # the CPU frame of the timed configuration over the reference rows:
            # the oracle at 64 spp on the GPU frame's own pools
            g = np.load(FP64_REFS)
            r0, r1 = (int(x) for x in g["c1_rows"])
            bpool = ctx.mrg_pool((r1 - r0) * W, spp * r["max_bounces"], seed=r["seed"], pixel0=r0 * W)
            t0 = time.perf_counter()
            band = orc.render(sc.camera, r, bpool, r0, r1)
            band_s = time.perf_counter() - t0
            scene.render_device(sc.camera, r, out.data_ptr())
            gpu_band = out.cpu().numpy()[r0:r1]
            full = np.zeros((H, W, 3), np.float32)
            full[r0:r1] = band
            line["rmse"]["cpu_frame"] = fp64_rmse(full, "c1", spp)["value"]
            line["rmse"]["cpu_frame_equals_gpu"] = bool(np.array_equal(band, gpu_band))
            line["rmse"]["cpu_frame_seconds"] = band_s
        orc.close()
    scene.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gbpt(args, rank, world)


if __name__ == "__main__":
    main()
