"""SPPM throughput benchmark (one JSON line on rank 0).

Headline workload (N=1 per GPU): the Cornell box of the 1024x1024 configuration -- unit cube, five
Lambertian walls, 0.25x0.25 ceiling light of emission 15, two 64x32 UV spheres (mirror, diffuse
0.73), 7,948 triangles -- rendered at 1024x1024 with 2^20 photon slots per pass, alpha 0.7, initial
radius 0.5% of the scene diagonal, the reference's xorshift seeding, plain FP32 (the reference's
precision).  A step is one SPPM pass (m_display); an eye pass runs every 10th pass, as in the
reference.  Data are synthetic (generated geometry); the reference publishes no number for this
workload.

  value     emitted photons per second (10^6), device-timed with CUDA events over K passes, state
            resident in HBM; the pass's working set (~190 MB) exceeds the 129 MB L2, so no flush.
  e2e       the same metric through the public API with host buffers: every step sets the camera
            (host->device), runs one pass and reads the linear radiance image back (device->host)
            into one of two page-locked buffers, the copy of step i running beside pass i+1.
  roofline  the photon-trace kernel's algorithmic bytes against the measured HBM copy bandwidth,
            with the DRAM traffic from the committed ncu summary beside it.
  cpu_baseline  the CPU oracle (C restatement of the shaders, OpenMP) on the host cores.
  rmse_vs_fp64  the radiance image's error against the double-precision oracle run with the same
            seed and random sequence for the same passes (precision error alone).
  full_config   the whole configuration (1000 passes) end to end: one sppm_run_passes call and one
            sppm_read_image.

The same line carries the other configurations (each can be skipped, and most are the headline of
their own --workload run):
  mixed        the headline workload on the mixed-precision path (4-wide quantised BVH, FP16 slot
               records, double-float statistics)                       (--no-mixed)
  batched      64 seeded Cornell variants advanced as one batch, FP32 and mixed, against the plain
               FP32 single-job path looped over the same jobs           (--no-batched; --workload batched)
  large        the 4.1M-triangle displaced sphere + heightfield at 1920x1080, 2^21 photons per pass,
               FP32 and mixed, BVH built on the GPU                    (--no-large; --workload large)
  serving      Poisson arrivals into the continuous-batching server, each request's target pass
               count from a target RMSE through the convergence calibration (--no-serving)
  convergence  the 256x256 workload after 64 passes against the committed converged FP64 reference

--impl reference: the reference's GLSL pipeline cannot run on this machine (no OpenGL stack), so the
reference arm times the CPU restatement of the reference's shader path (the oracle) on all host
cores, on the scene the reference's own host code built, a bounded number of passes; it never
loads the product library.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "SPPM Mphotons/s + Mrays/s at fixed RMSE vs FP64 oracle, plain vs batched"
WORKLOAD = {"workload": "cornell-1024", "image": "1024x1024", "photons_per_pass": 2 ** 20, "triangles": 7948,
            "passes_in_config": 1000, "alpha": 0.7, "radius": "0.5% of scene diagonal", "eye_pass_every": 10}
QUALITY_PASSES = 21  # two eye passes (frames 0, 10, 20)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def image_buffers(r) -> list:
    """The two page-locked host images a streaming caller reuses (allocated once, before timing)."""
    import glslppm_gb300 as g
    return [g.pinned_empty((r.height, r.width, 3), np.float32) for _ in range(2)]


def stream_frames(r, cam, steps: int, bufs: list) -> None:
    """`steps` end-to-end steps through the public API: camera up, one pass, the radiance image
    down into one of the caller's two page-locked buffers (the copy of a step overlaps the next
    pass); returns when the last image is in host memory."""
    from glslppm_gb300 import native as N

    tickets = [0, 0]
    for i in range(steps):
        k = i & 1
        if tickets[k]:
            r.image_wait(tickets[k])
        r.set_camera(cam)
        r.run_passes(1)
        tickets[k] = r.read_image_async(bufs[k], N.IMAGE_RADIANCE)
    r.synchronize()


def full_config_run(r, passes: int) -> dict:
    """The whole configuration end to end through the public API: one sppm_run_passes(passes) and
    one sppm_read_image of the result, wall-clock timed from the call to the image in host memory."""
    from glslppm_gb300 import native as N
    r.synchronize()
    f0 = r.frame_info()
    t0 = time.perf_counter()
    r.run_passes(passes)
    img = r.read_image(N.IMAGE_RADIANCE)
    dt = time.perf_counter() - t0
    f1 = r.frame_info()
    assert np.isfinite(img).all()
    ph = f1.photons_emitted - f0.photons_emitted
    return {"passes": passes, "seconds": round(dt, 4), "mphotons_per_s": round(ph / dt / 1e6, 3),
            "mrays_per_s": round(((f1.photon_segments + f1.eye_segments) - (f0.photon_segments + f0.eye_segments))
                                 / dt / 1e6, 3),
            "note": "one sppm_run_passes call and one sppm_read_image, host wall clock", "_image": img}


def converged_cornell1024(dev: int, passes: int) -> tuple[np.ndarray, float]:
    """A converged image of the headline workload's scene and camera, rendered on the GPU: the
    mixed path with the counting-sort grid (whose images are within 2e-4 of the FP64 oracle's grid
    estimator on the same random sequence) with an eye pass every pass, `passes` passes of 2^20
    photons from each of two seeds no other run uses, averaged.  SPPM converges to the same
    pixel-filtered radiance for any estimator and eye-pass interval.  Returns the image and its
    estimated relative error (half the two runs' relative difference)."""
    from glslppm_gb300 import native as N
    imgs = []
    for seed in (7, 11):
        r = make_renderer(dev, precision=N.PRECISION_MIXED, eye_pass_interval=1, flags=N.FLAG_PHOTON_GRID,
                          seed=seed)[0]
        r.run_passes(passes)
        imgs.append(r.read_image().astype(np.float64))
        r.close()
    return 0.5 * (imgs[0] + imgs[1]), rel_rmse(imgs[0], imgs[1]) / 2.0


def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,timestamp")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = None
        self.window = None

    def __enter__(self):
        try:
            self.out = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
            # wait (bounded) for the first sample so that the timed region is covered
            t0 = time.time()
            while time.time() - t0 < 5.0 and self.out.tell() == 0:
                time.sleep(0.05)
        except Exception:
            self.proc = None
        return self

    def mark(self, start: float, end: float):
        """Wall-clock window of the timed region; samples outside it are ignored."""
        self.window = (start, end)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.out.seek(0)
        rows = [r.split(", ") for r in self.out.read().strip().splitlines() if r.strip()]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        import datetime
        inside = []
        for r in rows:
            try:
                ts = datetime.datetime.strptime(r[9].strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except (ValueError, IndexError):
                ts = None
            if self.window is None or ts is None or (self.window[0] - 0.06 <= ts <= self.window[1] + 0.06):
                inside.append(r)
        if len(inside) >= 2:
            rows = inside
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for name, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def profile_traffic(kernel: str, workload: str = "cornell1024"):
    """Per-launch DRAM traffic of `kernel` on a workload, from the committed ncu summary
    (profiles/<kernel>_<workload>.md; the large-mesh summary covers both traversal kernels)."""
    name = f"{kernel}_{workload}.md" if workload == "cornell1024" else f"k_trace_photons_{workload}.md"
    p = REPO / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                if kernel == "k_trace_photons4" and workload != "cornell1024":
                    return float(line.split("k_trace_photons4:", 1)[1].split(")")[0])
                return float(line.split(":", 1)[1].split()[0])
            except (ValueError, IndexError):
                return None
    return None


def cornell_mesh():
    """The Cornell box as the product's host code loads it: the generated scene written as OBJ/MTL,
    read by the OBJ loader (the reference's loading rules) and given the exact-SAH BVH -- the same
    arrays, word for word, as the reference's own host code makes of that OBJ
    (tests/golden/cornell_box_scene.npz, which the CPU reference arm renders)."""
    import glslppm_gb300 as g
    from glslppm_gb300 import scenes
    sc = scenes.cornell_box()
    with tempfile.TemporaryDirectory() as td:
        mesh = g.Mesh.load_obj(str(sc.write_obj(Path(td) / "cornell_box.obj"))).build_bvh()
    return sc, mesh


def make_renderer(device: int, precision: int = 0, eye_pass_interval: int = 10, flags: int = 0, seed: int = 0):
    import glslppm_gb300 as g
    sc, mesh = cornell_mesh()
    cfg = g.default_config(1024, radius_rule=1, radius_fraction=0.005, precision=precision,
                           eye_pass_interval=eye_pass_interval, seed=seed)
    cfg.flags |= flags
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 1024, 1024, sc.fov)
    r = g.Renderer(cfg, device=device)
    r.upload_scene(mesh)
    r.set_camera(cam)
    return r, mesh, cfg, cam


def headline_config(precision: str, eye_pass_interval: int, world: int) -> dict:
    """The `config` of the headline line, identical for the GPU arm and the CPU reference arm."""
    return dict(WORKLOAD, precision=precision, l2="working set > 129 MB L2 (no flush)",
                eye_pass_every=eye_pass_interval, parallelism=f"replicas x{world}")


def autotune(ctx, args, cycles: int):
    """The library's launch-shape autotuner (Renderer/Batch.autotune) on the job's first passes,
    before the warm-up; the shapes chosen go into the line's config (None with --no-autotune)."""
    if args.tuning:  # fixed shapes (e.g. the ones a tuner chose in an earlier run): no tuner passes
        ctx.set_tuning(**json.loads(args.tuning))
        return ctx.get_tuning().as_dict()
    if args.no_autotune:
        return None
    best, _ = ctx.autotune(cycles)
    return best.as_dict()


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_baseline_run(max_seconds: float = 25.0, max_frames: int | None = None, warmup: int = 0):
    """The CPU oracle (the C restatement of the reference's shaders, OpenMP over all host threads)
    on the same workload, a bounded number of passes after `warmup` untimed ones.  The scene, its
    BVH and the camera are those the reference's own host code (mesh.cpp, bvh.cpp, camera.cpp) made
    of the Cornell box OBJ (tests/golden/cornell_box_scene.npz); the product library is not loaded."""
    from oracle.binding import Oracle
    from oracle.structs import RADIUS_DIAGONAL, camera_from_npz, default_config, scene_from_npz
    scene, d = scene_from_npz(REPO / "tests" / "golden" / "cornell_box_scene.npz")
    cfg = default_config(1024, radius_rule=RADIUS_DIAGONAL, radius_fraction=0.005)
    cam = camera_from_npz(d, 1024, 1024)
    o = Oracle(cfg, scene, cam)
    if warmup:
        o.run_frames(warmup)
    f0 = o.frame_info()
    t0 = time.perf_counter()
    frames = 0
    while True:
        o.run_frames(1)
        frames += 1
        el = time.perf_counter() - t0
        if el >= max_seconds or (max_frames and frames >= max_frames):
            break
    fi = o.frame_info()
    cores = os.cpu_count() or 1
    try:
        cores = len(os.sched_getaffinity(0))
    except Exception:
        pass
    return {"seconds": el, "frames": frames, "photons": int(fi.photons_emitted - f0.photons_emitted),
            "segments": int((fi.photon_segments + fi.eye_segments) - (f0.photon_segments + f0.eye_segments)),
            "cores": cores}


def run_reference(args, rank, world):
    if rank != 0:
        return
    budget = float(os.environ.get("SPPM_REFERENCE_SECONDS", "60"))
    res = cpu_baseline_run(max_seconds=budget, max_frames=args.steps, warmup=args.warmup)
    v = res["photons"] / res["seconds"] / 1e6
    sample = (f"{res['frames']} passes of the 1024x1024 / 2^20-photon workload after {args.warmup} untimed "
              f"ones, {res['seconds']:.1f} s")
    line = {
        "metric": METRIC,
        "value": round(v, 4), "unit": "Mphotons/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": res["frames"], "requested_steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000.0 * res["seconds"] / res["frames"], 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config("fp32", 10, world),
        "mrays_per_s": round(res["segments"] / res["seconds"] / 1e6, 4),
        "cpu_baseline": {"value": round(v, 4), "unit": "Mphotons/s", "cores": res["cores"], "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(v, 4), "unit": "Mphotons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's GLSL pipeline needs OpenGL, unavailable on this machine; this arm runs the CPU "
                "restatement of the reference's shaders (oracle/sppm_oracle.c) on the host cores, on the scene, BVH "
                "and camera the reference's own host code built (tests/golden/cornell_box_scene.npz); the product "
                "library is not loaded",
    }
    print(json.dumps(line), flush=True)


def roofline_of(cnt, trace_ms_per_launch: float, kernel: str, workload: str, peak: float, peak_kind: str,
                limiter: str) -> dict | None:
    """The traversal kernel against HBM: achieved = algorithmic bytes per launch (per photon segment
    64 + 32 V + 36 T: ray state, 32-byte nodes, 36-byte triangles; V, T from the traversal counters)
    over its event-timed duration; traffic = its DRAM bytes per launch from the committed ncu
    summary, also given as a rate (dram_gbs) -- the bandwidth the kernel really draws from HBM."""
    if not cnt or not trace_ms_per_launch:
        return None
    bpl = cnt["photon_segments"] / cnt["passes"] * (64 + 32 * cnt["nodes_per_segment"] + 36 * cnt["tris_per_segment"])
    sec = trace_ms_per_launch / 1000.0
    achieved = bpl / sec / 1e9
    traffic = profile_traffic(kernel, workload)
    out = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
           "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": kernel, "peak_kind": peak_kind,
           "nodes_per_segment": round(cnt["nodes_per_segment"], 2), "tris_per_segment": round(cnt["tris_per_segment"], 2),
           "algorithmic_bytes_per_launch": round(bpl), "launch_ms": round(trace_ms_per_launch, 4),
           "limiter": limiter}
    if traffic:
        out["dram_gbs"] = round(traffic / sec / 1e9, 1)
        out["dram_frac"] = round(traffic / sec / 1e9 / peak, 4)
    return out


LIMITER_L2 = {
    "k_trace_photons": ("dependent node loads and divergence: the BVH (3 MB) is L2-resident, so DRAM carries only the "
                        "ray queue (dram_frac); issue-active 68%, 13.8 of 32 lanes active, bins longest mean walk "
                        "first (profiles/k_trace_photons_cornell1024.md)"),
    "k_trace_photons4": ("instruction issue: the BVH (3 MB) is L2-resident, so DRAM carries only the ray queue "
                         "(dram_frac); issue-active 80%, 13.5 of 32 lanes active "
                         "(profiles/k_trace_photons4_cornell1024.md)"),
}
LIMITER_HBM = {
    "k_trace_photons": ("BVH and triangles (2.2 GB) exceed L2: node fetches reach DRAM; dependent-load latency at the "
                        "measured dram_frac, issue-active 42%, bins longest mean walk first "
                        "(profiles/k_trace_photons_largemesh.md)"),
    "k_trace_photons4": ("BVH and triangles (2.2 GB) exceed L2, but the 4-wide walk fetches a quarter as many nodes: "
                         "instruction issue, issue-active 72% at the measured dram_frac "
                         "(profiles/k_trace_photons_largemesh.md)"),
}


def measure_cornell(args, world: int, dev: int, precision: str, flags: int = 0) -> dict:
    """The headline workload at one precision (flags: e.g. the mixed path's counting-sort photon
    grid): autotuned launch shapes, W warm-up passes, K device-timed passes, a stage breakdown, the
    streamed end-to-end steps, the traversal roofline and the whole configuration end to end."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    prec = N.PRECISION_MIXED if precision == "mixed" else N.PRECISION_FP32
    r, mesh, cfg, cam = make_renderer(dev, precision=prec, eye_pass_interval=args.eye_pass_interval, flags=flags)
    K, W = args.steps, args.warmup
    P = cfg.photon_width * cfg.photon_height
    npix = cfg.width * cfg.height
    clocks = ClockSampler(dev).__enter__()
    # launch shapes chosen by the library's autotuner on the job's first passes (results do not
    # depend on them), then the warm-up passes (at least one eye pass) and an alignment to an
    # eye-pass boundary so the timed region holds exactly one eye pass per 10 passes
    tuning = autotune(r, args, cycles=2)
    r.run_passes(W)
    fi0 = r.frame_info()
    L = args.eye_pass_interval
    align = (L - fi0.frames % L) % L
    if align:
        r.run_passes(align)
    r.synchronize()
    fi0 = r.frame_info()
    # device-timed region (CUDA events on the library's stream; each frame replays its CUDA
    # graph); the photon traversal kernel carries its own events for the roofline
    r.time_stages(["photon_trace"])
    r.read_stage_times()
    barrier(world)
    t_wall = time.time()
    ms = r.time_passes(K)
    clocks.mark(t_wall, time.time())
    clocks.__exit__(None, None, None)
    tr_ms, tr_n = r.read_stage_times()["photon_trace"]
    r.time_stages([])
    fi1 = r.frame_info()
    photons = fi1.photons_emitted - fi0.photons_emitted
    segments = (fi1.photon_segments + fi1.eye_segments) - (fi0.photon_segments + fi0.eye_segments)
    t = max_over_ranks(ms / 1000.0, world)
    value = sum_over_ranks(photons, world) / t / 1e6
    mrays = sum_over_ranks(segments, world) / t / 1e6
    launches = fi1.kernel_launches - fi0.kernel_launches
    # per-stage breakdown (every stage timed) over a further 10-pass cycle, outside the timed region
    r.enable_stage_timing(True)
    r.read_stage_times()
    r.run_passes(10)
    stages = r.read_stage_times()
    r.enable_stage_timing(False)
    # end to end through the public API with (page-locked) host buffers
    E = args.e2e_steps
    bufs = image_buffers(r)
    r.synchronize()
    fe0 = r.frame_info()
    barrier(world)
    t0 = time.perf_counter()
    stream_frames(r, cam, E, bufs)
    te = max_over_ranks(time.perf_counter() - t0, world)
    fe1 = r.frame_info()
    e2e = sum_over_ranks(fe1.photons_emitted - fe0.photons_emitted, world) / te / 1e6
    # roofline of the photon traversal: algorithmic bytes of the exact walk of the same workload
    peak, peak_kind = measured_peaks()
    if prec == N.PRECISION_MIXED:
        r32 = make_renderer(dev, precision=N.PRECISION_FP32)[0]
        r32.run_passes(W)
        cnt = traversal_counters(r32)
        r32.close()
    else:
        cnt = traversal_counters(r)
    wide = prec == N.PRECISION_MIXED or bool((tuning or {}).get("wide_bvh"))
    kernel = "k_trace_photons4" if wide else "k_trace_photons"
    roof = roofline_of(cnt, tr_ms / tr_n if tr_n else 0.0, kernel, "cornell1024", peak, peak_kind, LIMITER_L2[kernel])
    r.close()
    # the whole configuration (1000 passes) end to end on a fresh context with the tuned shapes
    rf = make_renderer(dev, precision=prec, eye_pass_interval=args.eye_pass_interval, flags=flags)[0]
    if tuning:
        rf.set_tuning(**tuning)
    full = full_config_run(rf, WORKLOAD["passes_in_config"]) if not args.no_full_config else None
    rf.close()
    full_image = full.pop("_image") if full else None
    return {
        "value": round(value, 3), "ms_per_step": round(1000.0 * t / K, 4), "mrays_per_s": round(mrays, 3),
        "tuning": tuning,
        "stage_ms_per_launch": {k: round(v[0] / v[1], 4) for k, v in stages.items() if v[1]},
        "stage_bandwidth": stage_bandwidth(stages, npix, P, (fi1.photon_segments - fi0.photon_segments) / K, peak),
        "gpu_launches": int(launches),
        "e2e": {"value": round(e2e, 3), "unit": "Mphotons/s", "h2d_bytes_per_step": int(N.lib.sppm_camera_upload_bytes()),
                "d2h_bytes_per_step": int(npix * 3 * 4), "steps": E},
        "roofline": roof, "clocks": clocks.summary(), "full_config": full, "_full_image": full_image,
    }


# ---- image quality against the double-precision oracle ------------------------------------------
def rel_rmse(img, ref) -> float:
    a = np.asarray(img, np.float64)
    b = np.asarray(ref, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def error_stats(img, ref) -> dict:
    a = np.asarray(img, np.float64)
    rel = np.abs(a - ref) / np.maximum(np.abs(ref), 1e-6)
    return {"rel_rmse": round(rel_rmse(a, ref), 6), "p99_pixel_rel": round(float(np.percentile(rel, 99)), 5),
            "frac_pixels_within_1e-3": round(float(np.mean(rel <= 1e-3)), 4)}


def gpu_images(dev: int, cfg_fp32, scene_mesh, cam, passes: int, tuning: dict | None = None,
               paths=(("fp32", 0, 0), ("mixed", 1, 0))) -> dict:
    """The radiance images of fresh contexts after `passes` passes: paths = (name, precision, extra
    flags), by default FP32 and mixed."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    out = {}
    for name, prec, flags in paths:
        cfg = N.Config.from_buffer_copy(cfg_fp32)
        cfg.precision = prec
        cfg.flags |= flags
        r = g.Renderer(cfg, device=dev)
        r.upload_scene(scene_mesh)
        r.set_camera(cam)
        r.run_passes(passes)
        out[name] = r.read_image().astype(np.float64)
        r.close()
    return out


def quality_leg(quality_jobs: list) -> dict:
    """Part of the CPU leg (it runs the oracle, the checker): the double-precision oracle renders
    each workload's job with the same seed and random sequence (its GPURnd and cell hash are the
    single-precision ones) for the same passes as the GPU images, so the difference is the
    precision of the GPU paths, not Monte Carlo noise.  quality_jobs: (name, cfg, scene struct,
    camera, passes, {path: image})."""
    from oracle.binding import Oracle
    out = {}
    for name, cfg, scene, cam, passes, imgs in quality_jobs:
        t0 = time.perf_counter()
        o = Oracle(cfg, scene, cam, fp64=True)
        o.run_frames(passes)
        ref = o.read_image(0)
        o.close()
        out[name] = {"passes": passes, "oracle_seconds": round(time.perf_counter() - t0, 1),
                     **{path: error_stats(img, ref) for path, img in imgs.items()}}
    return out


def convergence(dev: int) -> dict | None:
    """The 256x256 workload after 64 passes (FP32 and mixed) against the committed converged FP64
    reference (tests/golden/c1_converged_fp64.npz: two 4096-pass FP64 oracle renders of other
    seeds), beside the calibration curve of tests/golden/convergence_c1.json."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    refp = REPO / "tests" / "golden" / "c1_converged_fp64.npz"
    calp = REPO / "tests" / "golden" / "convergence_c1.json"
    if not refp.exists() or not calp.exists():
        return None
    with np.load(refp) as z:
        ref = z["radiance"].astype(np.float64)
    cal = json.loads(calp.read_text())
    from tests.golden.fixtures import c1_camera_and_scene
    mesh, cam = c1_camera_and_scene()
    out = {"reference": {k: cal["reference"][k] for k in ("passes", "seeds", "photons", "photon_slots_per_pass",
                                                          "eye_pass_interval", "estimator", "estimated_rel_error")}}
    for name, prec, flags in (("fp32", N.PRECISION_FP32, 0), ("mixed", N.PRECISION_MIXED, 0),
                              ("grid", N.PRECISION_MIXED, N.FLAG_PHOTON_GRID)):
        cfg = g.default_config(256, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.005, precision=prec)
        cfg.flags |= flags
        r = g.Renderer(cfg, device=dev)
        r.upload_scene(mesh)
        r.set_camera(cam)
        # the whole 256x256 configuration (64 passes) end to end: one sppm_run_passes, one read
        full = full_config_run(r, 64)
        full.pop("_image")
        out[f"{name}_rel_rmse_after_64_passes"] = round(rel_rmse(r.read_image(), ref), 5)
        out[f"{name}_full_config_256"] = {k: full[k] for k in ("passes", "seconds", "mphotons_per_s")}
        r.close()
    out["calibration_rel_rmse_by_passes"] = cal["rel_rmse_by_passes"]
    out["grid_calibration_rel_rmse_by_passes"] = cal["grid_rel_rmse_by_passes"]
    # passes to reach 5% and 2% relative RMSE at the workload's own rate (one photon per pixel per
    # pass), from each estimator's fit
    out["passes_for_target"] = {f"{t:.0%}": {"winner": passes_for_target(t, 256 * 256, 1 << 16),
                                             "grid": passes_for_target(t, 256 * 256, 1 << 16, fit="grid_fit")}
                                for t in (0.05, 0.02)}
    return out


def noise_by_passes(dev: int, tuning: dict | None, checkpoints=(100, 1000)) -> dict:
    """Seed-to-seed image noise of the headline workload (1024x1024, 2^20 photons) on the mixed
    path with the reference's one-winner-per-slot estimator and with the counting-sort grid: the
    relative RMSE between renders of seeds 1 and 2 after each checkpoint, divided by sqrt(2) (the
    noise of one render), and the device time per pass of each."""
    from glslppm_gb300 import native as N
    out = {}
    for name, flags in (("winner", 0), ("grid", N.FLAG_PHOTON_GRID)):
        rs = [make_renderer(dev, precision=N.PRECISION_MIXED, flags=flags, seed=s)[0] for s in (1, 2)]
        for r in rs:
            if tuning:
                r.set_tuning(**tuning)
        done, noise = 0, {}
        for k in checkpoints:
            for r in rs:
                r.run_passes(k - done)
            done = k
            a, b = (r.read_image().astype(np.float64) for r in rs)
            noise[str(k)] = round(float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(((a + b) / 2) ** 2))) /
                                  math.sqrt(2.0), 5)
        ms = rs[0].time_passes(20) / 20
        for r in rs:
            r.close()
        out[name] = {"noise_by_passes": noise, "ms_per_pass": round(ms, 4)}
    return out


def passes_for_target(target_rmse: float, npix: int, photons_per_pass: int, cap: int = 1 << 20,
                      fit: str = "fit") -> int:
    """Pass count at which a job reaches `target_rmse` relative RMSE against a converged FP64
    reference, from the power-law fit over photons per pixel of tests/golden/convergence_c1.json
    (the 256x256 workload, one photon per pixel per pass; fit "fit" for the reference's estimator,
    "grid_fit" for the counting-sort grid's).  A job with more photons per pixel per pass still
    needs as many passes as the calibration workload: the gather radius shrinks once per pass, and
    with few passes its bias, not the photon noise, sets the error."""
    cal = json.loads((REPO / "tests" / "golden" / "convergence_c1.json").read_text())[fit]
    ppp = (cal["a"] / target_rmse) ** (1.0 / cal["b"])
    return int(min(cap, max(1, math.ceil(ppp), math.ceil(ppp * npix / photons_per_pass))))


def build_jobs(n_jobs: int, seed0: int = 0):
    """The batched workload's jobs: seeded Cornell variants, host BVH builds in parallel threads
    (the native build releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    import glslppm_gb300 as g
    from glslppm_gb300 import scenes
    specs = [scenes.cornell_variant(seed0 + i) for i in range(n_jobs)]
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        meshes = list(ex.map(lambda s: s.scene.to_mesh(), specs))
    jobs = []
    for s, m in zip(specs, meshes):
        cfg = g.default_config(s.width, height=s.height, photon_width=s.photon_width, photon_height=s.photon_height,
                               radius_rule=1, radius_fraction=0.005, seed=s.seed)
        cam = g.look_at(s.scene.camera_origin, s.scene.camera_lookat, s.width, s.height, s.scene.fov)
        jobs.append((s, m, cfg, cam))
    return jobs


BATCHED = {"workload": "cornell-variants-64", "jobs": 64, "triangles_per_job": "10k-500k (log-uniform)",
           "objects_per_job": "1-40 spheres/boxes", "images": "128^2/256^2/512^2/1024^2",
           "photons_per_pass_per_job": "2^14..2^19", "eye_pass_every": 10, "alpha": 0.7,
           "radius": "0.5% of scene diagonal"}


def run_batched(args, device: int, K: int, W: int, precision: int, jobs=None) -> dict:
    """The batched workload: 64 jobs advanced by one launch per stage (CUDA graph per pass)."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    t_setup = time.perf_counter()
    jobs = jobs or build_jobs(args.batch_jobs)
    b = g.Batch(precision=precision, max_jobs=len(jobs), device=device)
    ids = []
    for (_, m, cfg0, cam) in jobs:
        cfg = N.Config.from_buffer_copy(cfg0)
        cfg.precision = precision
        ids.append(b.add_job(cfg, m, cam))
    setup_s = time.perf_counter() - t_setup
    tuning = autotune(b, args, cycles=1)
    b.run_passes(W)
    b.synchronize()
    f0 = [b.frame_info(j) for j in ids]
    info_k0 = b.info().kernel_launches
    b.time_stages(["photon_trace"])
    b.read_stage_times()
    ms = b.time_passes(K)
    tr = b.read_stage_times()["photon_trace"]
    b.time_stages([])
    f1 = [b.frame_info(j) for j in ids]
    launches = b.info().kernel_launches - info_k0
    photons = sum(y.photons_emitted - x.photons_emitted for x, y in zip(f0, f1))
    segs = sum((y.photon_segments + y.eye_segments) - (x.photon_segments + x.eye_segments) for x, y in zip(f0, f1))
    info = b.info()
    batched = photons / (ms / 1000.0) / 1e6
    # end to end: every step sets each job's camera (host->device, one upload launch for all
    # jobs), runs one pass and reads each job's progress counters back (device->host)
    E = max(5, min(K, 30))
    cams = [cam for (_, _, _, cam) in jobs]
    fe0 = b.frame_infos(ids)
    t0 = time.perf_counter()
    for _ in range(E):
        b.set_cameras(ids, cams)
        b.run_passes(1)
        fe = b.frame_infos(ids)
    te = time.perf_counter() - t0
    e2e = sum(y.photons_emitted - x.photons_emitted for x, y in zip(fe0, fe)) / te / 1e6
    # per-stage breakdown over a further 10-pass cycle (every stage timed, outside the timed region)
    b.time_stages(list(N.STAGES))
    b.read_stage_times()
    b.run_passes(10)
    st = b.read_stage_times()
    b.time_stages([])
    cnt = b.traversal_counters(5) if precision == N.PRECISION_FP32 else None
    b.close()
    return {
        "config": dict(BATCHED, precision="mixed" if precision == N.PRECISION_MIXED else "fp32",
                       triangles_total=int(sum(s.scene.num_triangles for (s, _, _, _) in jobs)),
                       photon_slots_per_pass=int(info.photon_slots), pixels=int(info.pixels),
                       device_bytes=int(info.bytes_used)),
        "tuning": tuning,
        "value": round(batched, 3), "unit": "Mphotons/s", "mrays_per_s": round(segs / (ms / 1000.0) / 1e6, 3),
        "steps": K, "warmup": W, "ms_per_step": round(ms / K, 4),
        "photon_trace_ms_per_launch": round(tr[0] / max(tr[1], 1), 4),
        "stage_ms_per_launch": {k: round(v[0] / v[1], 4) for k, v in st.items() if v[1]},
        "traversal": ({"nodes_per_segment": round(cnt["nodes_per_segment"], 2),
                       "tris_per_segment": round(cnt["tris_per_segment"], 2)} if cnt else None),
        "e2e": {"value": round(e2e, 3), "unit": "Mphotons/s",
                "h2d_bytes_per_step": int(N.lib.sppm_camera_upload_bytes()) * len(ids),
                "d2h_bytes_per_step": int(N.lib.sppm_batch_frame_record_bytes()) * len(ids), "steps": E},
        "setup_seconds": round(setup_s, 2), "gpu_launches": int(launches),
        "_trace": tr, "_counters": cnt, "_photons": photons, "_ms": ms,
    }


def plain_loop(args, device: int, jobs, K: int, W: int) -> dict:
    """The plain FP32 single-job path looped over the same jobs: each job's device time per pass,
    summed."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    loop_ms, loop_photons = 0.0, 0
    for (s, m, cfg0, cam) in jobs:
        cfg = N.Config.from_buffer_copy(cfg0)
        cfg.precision = N.PRECISION_FP32
        r = g.Renderer(cfg, device=device)
        r.upload_scene(m)
        r.set_camera(cam)
        r.run_passes(W)
        r.synchronize()
        a = r.frame_info()
        k = max(10, K // 4)
        t = r.time_passes(k)
        z = r.frame_info()
        loop_ms += t / k
        loop_photons += (z.photons_emitted - a.photons_emitted) / k
        r.close()
    return {"value": round(loop_photons / (loop_ms / 1000.0) / 1e6, 3), "unit": "Mphotons/s",
            "ms_per_pass_all_jobs": round(loop_ms, 4),
            "note": "plain FP32 single-job contexts run one after another, device time per pass summed"}


def batched_section(args, device: int, W: int, quality_jobs: list) -> dict:
    """Batched FP32 and mixed against the plain FP32 loop; the largest job's images for the
    quality leg."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    jobs = build_jobs(args.batch_jobs)
    fp32 = run_batched(args, device, args.batch_steps, W, N.PRECISION_FP32, jobs)
    mixed = run_batched(args, device, args.batch_steps, W, N.PRECISION_MIXED, jobs) if not args.no_mixed else None
    loop = plain_loop(args, device, jobs, args.batch_steps, W)
    out = {"fp32": {k: v for k, v in fp32.items() if not k.startswith("_")}, "plain_loop": loop,
           "speedup_vs_plain_loop": {"fp32": round(fp32["value"] / loop["value"], 3)},
           "target": "batched mixed >= 10x the plain FP32 loop at equal RMSE (<= 1% relative vs the FP64 oracle)"}
    if mixed:
        out["mixed"] = {k: v for k, v in mixed.items() if not k.startswith("_")}
        out["speedup_vs_plain_loop"]["mixed"] = round(mixed["value"] / loop["value"], 3)
    if not args.no_quality:
        i = max(range(len(jobs)), key=lambda j: jobs[j][0].scene.num_triangles)
        s, m, cfg, cam = jobs[i]
        imgs = gpu_images(device, cfg, m, cam, QUALITY_PASSES)
        quality_jobs.append(("batched_largest_job", cfg, m.scene(), cam, QUALITY_PASSES, imgs))
        out["quality_job"] = {"index": i, "triangles": s.scene.num_triangles, "image": f"{cfg.width}x{cfg.height}",
                              "photons_per_pass": cfg.photon_width * cfg.photon_height,
                              "note": "a batch job's state equals its single-job context's bit for bit "
                                      "(tests/test_gpu_batch.py), so its images come from single contexts"}
    out["_fp32"], out["_mixed"] = fp32, mixed
    return out


SERVING = {"workload": "serving-poisson", "scene_pool": "seeded Cornell variants as in the batched workload",
           "camera": "random origin within 0.15 of the default, looking at the box centre",
           "memory_budget_gb": 180, "eye_pass_every": 10}


def run_serving(args, device: int, tuning: dict | None = None) -> dict:
    """Poisson arrivals of render requests into the continuous-batching server.  Each request's
    target is a relative RMSE against a converged FP64 reference, turned into a pass count for its
    own resolution and photon budget through the convergence calibration of the 256x256 workload
    (tests/golden/convergence_c1.json).  Per arrival rate: p50/p99 time to target, aggregate
    Mphotons/s, and the achieved RMSE of sampled requests against a reference rendered with 16x
    their passes from another seed."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    rng = np.random.default_rng(12345)
    pool = build_jobs(args.serve_pool)
    prec = N.PRECISION_MIXED if args.precision == "mixed" else N.PRECISION_FP32
    rates = [float(x) for x in args.serve_rates.split(",")]
    rows = []
    for lam in rates:
        # launch shapes: those the batched workload's autotuner chose (same scene distribution)
        srv = g.Server(precision=prec, max_jobs=256, memory_budget=180 << 30, passes_per_step=args.serve_passes_per_step,
                       device=device,
                       tuning=tuning)
        n = int(min(args.serve_requests, max(8, math.ceil(lam * args.serve_window))))
        gaps = rng.exponential(1.0 / lam, n)
        reqs = []
        for i in range(n):
            s, m, cfg0, _ = pool[int(rng.integers(len(pool)))]
            cfg = g.default_config(cfg0.width, height=cfg0.height, photon_width=cfg0.photon_width,
                                   photon_height=cfg0.photon_height, radius_rule=1, radius_fraction=0.005,
                                   seed=int(rng.integers(1, 1 << 30)), precision=prec)
            o = np.array(s.scene.camera_origin) + rng.uniform(-0.15, 0.15, 3)
            cam = g.look_at(tuple(o), (0.5, 0.5, 0.5), cfg.width, cfg.height, s.scene.fov)
            tp = passes_for_target(args.serve_target_rmse, cfg.width * cfg.height, cfg.photon_width * cfg.photon_height)
            reqs.append((cfg, m, cam, tp))
        t0 = time.perf_counter()
        tickets = []
        due = 0.0
        for (cfg, m, cam, tp), gap in zip(reqs, gaps):
            due += gap
            d = due - (time.perf_counter() - t0)
            if d > 0:
                time.sleep(d)
            tickets.append(srv.submit(cfg, m, cam, tp))
        infos = [srv.wait(t, timeout=3600) for t in tickets]
        st = srv.stats()
        # achieved error of sampled requests: the request's image against the same job rendered
        # with 16x its passes from another seed (the FP32 path's precision error against the FP64
        # oracle is ~1e-3, far below the targets)
        sampled = []
        for k in rng.choice(len(tickets), size=min(args.serve_sample, len(tickets)), replace=False):
            if infos[k].state != N.REQUEST_DONE:
                continue
            img = srv.fetch_image(tickets[k])
            cfg, m, cam, tp = reqs[k]
            rc = N.Config.from_buffer_copy(cfg)
            rc.seed = cfg.seed ^ 0x5A5A5A5A
            rr = g.Renderer(rc, device=device)
            rr.upload_scene(m)
            rr.set_camera(cam)
            rr.run_passes(min(16 * tp, 1 << 16))
            sampled.append({"image": f"{cfg.width}x{cfg.height}", "photons_per_pass": cfg.photon_width * cfg.photon_height,
                            "target_passes": tp, "rel_rmse": round(rel_rmse(img, rr.read_image()), 4)})
            rr.close()
        srv.close()
        ok = [i for i in infos if i.state == N.REQUEST_DONE]
        ttt = np.array([i.t_done - i.t_submit for i in ok])
        span = max(i.t_done for i in ok) - min(i.t_submit for i in infos)
        rows.append({"rate_per_s": lam, "requests": n, "completed": len(ok),
                     "p50_time_to_target_s": round(float(np.percentile(ttt, 50)), 4),
                     "p99_time_to_target_s": round(float(np.percentile(ttt, 99)), 4),
                     "mean_queue_wait_s": round(float(np.mean([i.t_admit - i.t_submit for i in ok])), 4),
                     "mphotons_per_s": round(sum(i.photons_emitted for i in ok) / span / 1e6, 3),
                     "busy_fraction": round(st.busy_seconds / span, 3),
                     "mean_target_passes": round(float(np.mean([r[3] for r in reqs])), 1),
                     "sampled_achieved_rmse": sampled})
    return {"config": dict(SERVING, precision=args.precision, rates=args.serve_rates,
                           passes_per_step=args.serve_passes_per_step,
                           target_rel_rmse=args.serve_target_rmse,
                           requests_per_rate=f"min({args.serve_requests}, rate x {args.serve_window} s)",
                           target_passes="from the target RMSE through tests/golden/convergence_c1.json's fit, "
                                         "per request resolution and photon budget", tuning=tuning),
            "by_rate": rows}


LARGE = {"workload": "large-mesh", "triangles": "4.1M (displaced geodesic sphere 2.01M + heightfield 2.09M)",
         "image": "1920x1080", "photons_per_pass": 2 ** 21, "passes_in_config": 200, "materials": 4005,
         "lights": "4 quads, emission 5-20", "radius": "0.5% of scene diagonal", "eye_pass_every": 10,
         "bvh": "built on the GPU by locally-ordered clustering (PLOC) of Morton-sorted triangles"}


def large_scene(local: int):
    import glslppm_gb300 as g
    from glslppm_gb300 import scenes
    t0 = time.perf_counter()
    sc = scenes.large_mesh(1)
    t_gen = time.perf_counter() - t0
    mesh = g.Mesh.from_arrays(sc.positions, sc.material_ids, sc.material_array(), sc.normals)
    t1 = time.perf_counter()
    mesh.build_bvh(gpu=True, device=local)
    t_bvh = time.perf_counter() - t1
    return sc, mesh, {"generate": round(t_gen, 2), "gpu_bvh_build": round(t_bvh, 3)}


def large_config(prec: int):
    import glslppm_gb300 as g
    return g.default_config(1920, height=1080, photon_width=2048, photon_height=1024, radius_rule=1,
                            radius_fraction=0.005, precision=prec)


def run_large(args, world, local, K, W, prec: int, sc, mesh, setup: dict) -> dict:
    """The large-mesh workload at one precision (every rank measures; rank 0 prints)."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    cfg = large_config(prec)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 1920, 1080, sc.fov)
    r = g.Renderer(cfg, device=local)
    t2 = time.perf_counter()
    r.upload_scene(mesh)
    t_up = time.perf_counter() - t2
    r.set_camera(cam)
    clocks = ClockSampler(local).__enter__()
    tuning = autotune(r, args, cycles=1)
    r.run_passes(W)
    fi0 = r.frame_info()
    align = (10 - fi0.frames % 10) % 10
    if align:
        r.run_passes(align)
    r.synchronize()
    fi0 = r.frame_info()
    r.time_stages(["photon_trace"])
    r.read_stage_times()
    barrier(world)
    t_wall = time.time()
    ms = r.time_passes(K)
    clocks.mark(t_wall, time.time())
    clocks.__exit__(None, None, None)
    tr_ms, tr_n = r.read_stage_times()["photon_trace"]
    r.time_stages([])
    fi1 = r.frame_info()
    launches = fi1.kernel_launches - fi0.kernel_launches
    t = max_over_ranks(ms / 1000.0, world)
    photons = sum_over_ranks(fi1.photons_emitted - fi0.photons_emitted, world)
    segs = sum_over_ranks((fi1.photon_segments + fi1.eye_segments) - (fi0.photon_segments + fi0.eye_segments), world)
    value = photons / t / 1e6
    r.enable_stage_timing(True)
    r.read_stage_times()
    r.run_passes(10)
    stages = r.read_stage_times()
    r.enable_stage_timing(False)
    # end to end: camera up, one pass, radiance image down (pinned host buffer)
    E = max(5, min(K, 20))
    bufs = image_buffers(r)
    r.synchronize()
    fe0 = r.frame_info()
    te0 = time.perf_counter()
    stream_frames(r, cam, E, bufs)
    te = max_over_ranks(time.perf_counter() - te0, world)
    fe1 = r.frame_info()
    e2e = sum_over_ranks(fe1.photons_emitted - fe0.photons_emitted, world) / te / 1e6
    peak, peak_kind = measured_peaks()
    if prec == N.PRECISION_FP32:
        cnt = traversal_counters(r)
    else:
        r32 = g.Renderer(large_config(N.PRECISION_FP32), device=local)
        r32.upload_scene(mesh)
        r32.set_camera(cam)
        r32.run_passes(W)
        cnt = traversal_counters(r32)
        r32.close()
    wide = prec == N.PRECISION_MIXED or bool((tuning or {}).get("wide_bvh"))
    kname = "k_trace_photons4" if wide else "k_trace_photons"
    roof = roofline_of(cnt, tr_ms / tr_n if tr_n else 0.0, kname, "largemesh", peak, peak_kind, LIMITER_HBM[kname])
    r.close()
    full = None
    if not args.no_full_config:
        rf = g.Renderer(cfg, device=local)
        rf.upload_scene(mesh)
        rf.set_camera(cam)
        if tuning:
            rf.set_tuning(**tuning)
        full = full_config_run(rf, LARGE["passes_in_config"])
        full.pop("_image")
        rf.close()
    return {
        "metric": METRIC, "value": round(value, 3), "unit": "Mphotons/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": round(1000.0 * t / K, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(LARGE, precision="mixed" if prec == N.PRECISION_MIXED else "fp32",
                       triangles_exact=sc.num_triangles, l2="BVH + triangles 2.2 GB > 129 MB L2 (no flush)",
                       parallelism=f"replicas x{world}"),
        "tuning": tuning, "mrays_per_s": round(segs / t / 1e6, 3),
        "stage_ms_per_launch": {k: round(v[0] / v[1], 4) for k, v in stages.items() if v[1]},
        "setup_seconds": dict(setup, upload=round(t_up, 2)), "gpu_launches": int(launches),
        "e2e": {"value": round(e2e, 3), "unit": "Mphotons/s", "h2d_bytes_per_step": int(N.lib.sppm_camera_upload_bytes()),
                "d2h_bytes_per_step": int(cfg.width * cfg.height * 12), "steps": E},
        "roofline": roof, "cpu_baseline": None, "clocks": clocks.summary(), "full_config": full,
    }


def large_section(args, world, local, W, quality_jobs: list) -> dict:
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    sc, mesh, setup = large_scene(local)
    out = {"fp32": run_large(args, world, local, args.large_steps, W, N.PRECISION_FP32, sc, mesh, setup)}
    if not args.no_mixed:
        out["mixed"] = run_large(args, world, local, args.large_steps, W, N.PRECISION_MIXED, sc, mesh, setup)
    if not args.no_quality:
        cam = g.look_at(sc.camera_origin, sc.camera_lookat, 1920, 1080, sc.fov)
        cfg = large_config(N.PRECISION_FP32)
        imgs = gpu_images(local, cfg, mesh, cam, args.large_quality_passes)
        quality_jobs.append(("large", cfg, mesh.scene(), cam, args.large_quality_passes, imgs))
        out["_keep"] = (sc, mesh)  # the oracle reads the mesh's arrays in the CPU leg
    return out


def public(d: dict | None) -> dict | None:
    return None if d is None else {k: v for k, v in d.items() if not k.startswith("_")}


def run_gpu(args, rank, world, local):
    """The default line: the headline workload (plain FP32) with every other configuration beside it."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    if world > 1 or rank != 0:
        args.no_quality = True  # replicas: the image-error legs run once, on a single GPU
    quality_jobs: list = []
    if args.photon_grid and args.precision != "mixed":
        raise SystemExit("--photon-grid applies to --precision mixed")
    head = measure_cornell(args, world, local, args.precision, flags=N.FLAG_PHOTON_GRID if args.photon_grid else 0)
    out = {
        "metric": METRIC, "value": head["value"], "unit": "Mphotons/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(args.precision, args.eye_pass_interval, world),
        **{k: head[k] for k in ("tuning", "mrays_per_s", "stage_ms_per_launch", "stage_bandwidth", "gpu_launches",
                                "e2e", "roofline", "clocks", "full_config")},
        "cpu_baseline": None,
    }
    full_images = {args.precision: head["_full_image"]}
    if args.photon_grid:
        out["config"]["estimator"] = "counting-sort photon grid (every photon within the radius)"
    if args.precision == "fp32" and not args.no_mixed:
        out["mixed"] = measure_cornell(args, world, local, "mixed")
        full_images["mixed"] = out["mixed"].pop("_full_image")
        if not args.no_grid:
            gr = measure_cornell(args, world, local, "mixed", flags=N.FLAG_PHOTON_GRID)
            full_images["grid"] = gr.pop("_full_image")
            out["grid"] = {k: gr[k] for k in ("value", "ms_per_step", "mrays_per_s", "tuning", "stage_ms_per_launch",
                                              "gpu_launches", "e2e", "clocks", "full_config")}
            out["grid"]["note"] = ("mixed path with the counting-sort photon grid (SPPM_FLAG_PHOTON_GRID): every photon "
                                   "within the radius instead of one winner per hash slot times its count")
            if rank == 0 and world == 1:
                out["grid"]["noise"] = noise_by_passes(local, out["mixed"].get("tuning"))
    if not args.no_quality:
        r, mesh, cfg, cam = make_renderer(local, precision=N.PRECISION_FP32, eye_pass_interval=args.eye_pass_interval)
        r.close()
        quality_jobs.append(("cornell-1024", cfg, mesh.scene(), cam, QUALITY_PASSES,
                             gpu_images(local, cfg, mesh, cam, QUALITY_PASSES)))
        if "grid" in out:
            gcfg = N.Config.from_buffer_copy(cfg)
            gcfg.flags |= N.FLAG_PHOTON_GRID
            quality_jobs.append(("cornell-1024-grid", gcfg, mesh.scene(), cam, QUALITY_PASSES,
                                 gpu_images(local, gcfg, mesh, cam, QUALITY_PASSES,
                                            paths=(("grid", N.PRECISION_MIXED, 0),))))
        out["_keep_mesh"] = mesh
    batch_tuning = None
    if not args.no_batched:
        bs = batched_section(args, local, args.warmup, quality_jobs)
        batch_tuning = bs["fp32"]["tuning"]
        out["batched"] = public(bs)
    if not args.no_large:
        ls = large_section(args, world, local, args.warmup, quality_jobs)
        out["large"] = {k: {f: v[f] for f in ("value", "unit", "steps", "ms_per_step", "mrays_per_s", "config", "tuning",
                                               "stage_ms_per_launch", "setup_seconds", "e2e", "roofline", "full_config")}
                        for k, v in ls.items() if not k.startswith("_")}
        out["_keep_large"] = ls.get("_keep")
    if not args.no_serving:
        out["serving"] = run_serving(args, local, batch_tuning)
    if rank == 0 and world == 1 and not args.no_quality:
        out["convergence"] = convergence(local)
        if not args.no_full_config and all(v is not None for v in full_images.values()):
            # the whole 1024x1024 configuration's error: each path's image after its 1000 passes
            # against a converged image of the same scene and camera
            ref, ref_err = converged_cornell1024(local, args.converged_passes)
            out["full_config_rel_rmse"] = {
                **{k: round(rel_rmse(v, ref), 5) for k, v in full_images.items()},
                "passes": WORKLOAD["passes_in_config"],
                "reference": {"passes_per_seed": args.converged_passes, "seeds": [7, 11], "eye_pass_every": 1,
                              "path": "mixed + counting-sort grid (within 2e-4 of the FP64 oracle's grid estimator)",
                              "estimated_rel_error": round(ref_err, 5)}}
    # the CPU leg (rank 0, one GPU): the oracle timed as the CPU baseline, and as the checker, the
    # double-precision references of the image-error figures
    if rank == 0 and world == 1:
        if not args.no_cpu_baseline:
            res = cpu_baseline_run(max_seconds=args.cpu_seconds, warmup=3)
            out["cpu_baseline"] = {"value": round(res["photons"] / res["seconds"] / 1e6, 4), "unit": "Mphotons/s",
                                   "cores": res["cores"], "kind": "port",
                                   "sample": f"{res['frames']} passes of the same workload after 3 untimed ones, "
                                             f"{res['seconds']:.1f} s"}
        if quality_jobs:
            q = quality_leg(quality_jobs)
            note = ("radiance image after the stated passes against the FP64 oracle run with the same seed and "
                    "random sequence (precision error; Monte Carlo noise cancels)")
            if "cornell-1024" in q:
                out["rmse_vs_fp64"] = dict(q["cornell-1024"]["fp32"], passes=QUALITY_PASSES, note=note)
                if "mixed" in out:
                    out["mixed"]["rmse_vs_fp64"] = dict(q["cornell-1024"]["mixed"], passes=QUALITY_PASSES)
            if "cornell-1024-grid" in q and "grid" in out:
                out["grid"]["rmse_vs_fp64"] = dict(q["cornell-1024-grid"]["grid"], passes=QUALITY_PASSES,
                                                   note="against the FP64 oracle's grid estimator, same seed and sequence")
            if "batched_largest_job" in q and "batched" in out:
                out["batched"]["rmse_vs_fp64"] = q["batched_largest_job"]
            if "large" in q and "large" in out:
                out["large"]["rmse_vs_fp64"] = q["large"]
    for k in [k for k in out if k.startswith("_")]:
        del out[k]
    if rank == 0:
        print(json.dumps(out), flush=True)
    return out


def run_batched_line(args, rank, world, local):
    """--workload batched: the batched workload as the headline JSON line."""
    from glslppm_gb300 import native as N
    prec = N.PRECISION_MIXED if args.precision == "mixed" else N.PRECISION_FP32
    clocks = ClockSampler(local).__enter__()
    jobs = build_jobs(args.batch_jobs)
    barrier(world)
    t_wall = time.time()
    res = run_batched(args, local, args.steps, args.warmup, prec, jobs)
    clocks.mark(t_wall, time.time())
    clocks.__exit__(None, None, None)
    loop = plain_loop(args, local, jobs, args.steps, args.warmup)
    t = max_over_ranks(res["_ms"] / 1000.0, world)
    value = sum_over_ranks(res["_photons"], world) / t / 1e6
    peak, peak_kind = measured_peaks()
    tr_ms, tr_n = res["_trace"]
    wide = prec == N.PRECISION_MIXED or bool((res["tuning"] or {}).get("wide_bvh"))
    roof = roofline_of(res["_counters"], tr_ms / tr_n if tr_n else 0.0,
                       "k_trace_photons4" if wide else "k_trace_photons", "batched64", peak, peak_kind,
                       "dependent-load latency over 64 jobs' BVHs (5.8M triangles)")
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mphotons/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000.0 * t / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(res["config"], l2="working set > 129 MB L2 (no flush)", parallelism=f"replicas x{world}"),
            "tuning": res["tuning"], "mrays_per_s": res["mrays_per_s"], "plain_loop": loop,
            "speedup_vs_plain_loop": round(res["value"] / loop["value"], 3),
            "photon_trace_ms_per_launch": res["photon_trace_ms_per_launch"],
            "stage_ms_per_launch": res["stage_ms_per_launch"], "traversal": res["traversal"],
            "gpu_launches": res["gpu_launches"], "e2e": res["e2e"], "roofline": roof, "cpu_baseline": None,
            "clocks": clocks.summary(), "setup_seconds": res["setup_seconds"],
        }
        print(json.dumps(line), flush=True)


def run_large_line(args, rank, world, local):
    """--workload large: the large-mesh scene at 1920x1080 with 2^21 photons per pass."""
    from glslppm_gb300 import native as N
    prec = N.PRECISION_MIXED if args.precision == "mixed" else N.PRECISION_FP32
    sc, mesh, setup = large_scene(local)
    line = run_large(args, world, local, args.steps, args.warmup, prec, sc, mesh, setup)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_serving_line(args, rank, world, local):
    """--workload serving: the serving sweep; value = aggregate Mphotons/s at the highest rate."""
    clocks = ClockSampler(local).__enter__()
    t_wall = time.time()
    sv = run_serving(args, local)
    clocks.mark(t_wall, time.time())
    clocks.__exit__(None, None, None)
    top = sv["by_rate"][-1]
    value = sum_over_ranks(top["mphotons_per_s"], world)
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mphotons/s", "n_gpus": world, "steps": top["requests"],
            "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(sv["config"], parallelism=f"replicas x{world}"),
            "serving": sv["by_rate"],
            "e2e": {"value": round(value, 3), "unit": "Mphotons/s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": None,
                    "note": "requests submitted and images fetched through the server API; a step is a request"},
            "roofline": None, "cpu_baseline": None, "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)


def stage_bandwidth(stages: dict, npix: int, photon_slots: int, segments_per_pass: float, peak: float) -> dict:
    """Algorithmic bytes over event-timed launch duration for the memory-bound stages:
    gather + update 472 B per pixel (40 B hit point, 8 x (8 B slot + 36 B photon), 80 B of
    statistics read and written), photon store + hash insert 28 B per stored segment (16 B position
    and validity, 4 B key, 8 B atomics) plus the 48-byte photon record written, ray binning 12 B
    per queued ray."""
    out = {}
    units = {"gather": (npix, 472.0), "photon_store": (segments_per_pass, 28.0 + 48.0),
             "ray_bins": (segments_per_pass, 12.0)}
    for name, (n, per) in units.items():
        ms, cnt = stages.get(name, (0.0, 0))
        if cnt and ms > 0:
            gbs = n * per / (ms / cnt / 1000.0) / 1e9
            out[name] = {"bytes_per_unit": per, "units": int(n), "achieved_gbs": round(gbs, 1),
                         "frac": round(gbs / peak, 4)}
    return out


def traversal_counters(r):
    """Mean nodes visited and triangles tested per photon segment (counting kernel variant)."""
    try:
        return r.traversal_counters(passes=10)
    except (AttributeError, NotImplementedError):
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "mixed"])
    ap.add_argument("--eye-pass-interval", type=int, default=10,
                    help="passes per eye pass of the headline workload (the reference's is 10; a larger "
                         "value measures what the eye pass costs)")
    ap.add_argument("--e2e-steps", type=int, default=100, help="streamed end-to-end steps of the headline workload")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-quality", action="store_true",
                    help="skip the image-error figures against the FP64 oracle (and the convergence figure)")
    ap.add_argument("--no-full-config", action="store_true", help="skip the whole-configuration end-to-end runs")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision figures beside the FP32 ones")
    ap.add_argument("--no-grid", action="store_true", help="skip the counting-sort photon grid's figures")
    ap.add_argument("--converged-passes", type=int, default=8192,
                    help="passes per seed of the converged 1024x1024 image the whole configuration is measured against")
    ap.add_argument("--photon-grid", action="store_true",
                    help="headline workload on the mixed path with the counting-sort photon grid (--precision mixed)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch shapes instead of autotuning them before the warm-up")
    ap.add_argument("--tuning", default=None,
                    help='fixed launch shapes as JSON, e.g. \'{"trace_refill_steps": 4, "unbinned_rays": 1}\' '
                         "(sppm_tuning fields; replaces the autotuner)")
    ap.add_argument("--workload", default="cornell-1024", choices=["cornell-1024", "batched", "serving", "large"],
                    help="the JSON line's headline workload; the default line also carries the other "
                         "configurations' summaries")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--large-steps", type=int, default=20)
    ap.add_argument("--large-quality-passes", type=int, default=3)
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=30)
    ap.add_argument("--serve-rates", default="1,10,50,100,200")
    ap.add_argument("--serve-requests", type=int, default=300, help="requests per rate (at most)")
    ap.add_argument("--serve-window", type=float, default=20.0,
                    help="arrival window per rate in seconds: a rate gets min(--serve-requests, rate x window)")
    ap.add_argument("--serve-target-rmse", type=float, default=0.10,
                    help="each request's target relative RMSE against a converged FP64 reference")
    ap.add_argument("--serve-sample", type=int, default=2, help="requests per rate whose achieved RMSE is measured")
    ap.add_argument("--serve-pool", type=int, default=32)
    ap.add_argument("--serve-passes-per-step", type=int, default=1,
                    help="passes the server runs between admissions (a job finishing within a step stops at its "
                         "own pass count)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "batched":
        run_batched_line(args, rank, world, local)
    elif args.workload == "serving":
        run_serving_line(args, rank, world, local)
    elif args.workload == "large":
        run_large_line(args, rank, world, local)
    else:
        run_gpu(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
