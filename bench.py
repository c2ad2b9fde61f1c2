"""SPPM throughput benchmark (one JSON line on rank 0).

Workload (N=1 per GPU): the Cornell box of the 1024x1024 configuration -- unit cube, five
Lambertian walls, 0.25x0.25 ceiling light of emission 15, two 64x32 UV spheres (mirror, diffuse
0.73), 7,948 triangles -- rendered at 1024x1024 with 2^20 photon slots per pass, alpha 0.7, initial
radius 0.5% of the scene diagonal, the reference's xorshift seeding.  A step is one SPPM pass
(m_display); an eye pass runs every 10th pass, as in the reference.  Data are synthetic (generated
geometry); the reference publishes no number for this workload.

  value   emitted photons per second (10^6), device-timed with CUDA events over K passes, state
          resident in HBM; the pass's working set (~190 MB) exceeds the 129 MB L2, so no flush.
  e2e     the same metric through the public API with host buffers: every step sets the camera
          (host->device), runs one pass and reads the linear radiance image back (device->host).
  roofline  the photon-trace kernel against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (C restatement of the shaders, OpenMP) on the host cores.

--impl reference: the reference's GLSL pipeline cannot run on this machine (no OpenGL stack), so the
reference arm times the CPU restatement of the reference's shader path (the oracle) on all host
cores, on the same workload, a bounded number of passes.
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

WORKLOAD = {"workload": "cornell-1024", "image": "1024x1024", "photons_per_pass": 2 ** 20, "triangles": 7948,
            "passes_in_config": 1000, "alpha": 0.7, "radius": "0.5% of scene diagonal", "eye_pass_every": 10}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


def profile_traffic(kernel: str):
    """Per-launch DRAM traffic of `kernel` on this workload, from its committed ncu summary."""
    p = REPO / "profiles" / f"{kernel}_cornell1024.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def make_renderer(device: int, precision: int = 0):
    import glslppm_gb300 as g
    from glslppm_gb300 import scenes
    sc = scenes.cornell_box()
    mesh = sc.to_mesh()
    cfg = g.default_config(1024, radius_rule=1, radius_fraction=0.005, precision=precision)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 1024, 1024, sc.fov)
    r = g.Renderer(cfg, device=device)
    r.upload_scene(mesh)
    r.set_camera(cam)
    return r, mesh, cfg, cam


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


def cpu_baseline_run(max_seconds: float = 25.0, max_frames: int | None = None):
    """The CPU oracle on the same workload, all host threads, a bounded number of passes."""
    import glslppm_gb300 as g
    from glslppm_gb300 import scenes
    from oracle.binding import Oracle
    sc = scenes.cornell_box()
    mesh = sc.to_mesh()
    cfg = g.default_config(1024, radius_rule=1, radius_fraction=0.005)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 1024, 1024, sc.fov)
    o = Oracle(cfg, mesh.scene(), cam)
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
    return {"seconds": el, "frames": frames, "photons": int(fi.photons_emitted),
            "segments": int(fi.photon_segments + fi.eye_segments), "cores": cores}


def run_reference(args, rank, world):
    if rank != 0:
        return
    budget = float(os.environ.get("SPPM_REFERENCE_SECONDS", "60"))
    res = cpu_baseline_run(max_seconds=budget, max_frames=args.steps)
    v = res["photons"] / res["seconds"] / 1e6
    line = {
        "metric": "SPPM Mphotons/s + Mrays/s at fixed RMSE vs FP64 oracle, plain vs batched",
        "value": round(v, 4), "unit": "Mphotons/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": res["frames"], "requested_steps": args.steps, "warmup": 0,
        "ms_per_step": round(1000.0 * res["seconds"] / res["frames"], 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(WORKLOAD, sample=f"first {res['frames']} passes from frame 0"),
        "mrays_per_s": round(res["segments"] / res["seconds"] / 1e6, 4),
        "cpu_baseline": {"value": round(v, 4), "unit": "Mphotons/s", "cores": res["cores"], "kind": "port",
                         "sample": f"{res['frames']} passes of the 1024x1024 / 2^20-photon workload from frame 0"},
        "e2e": {"value": round(v, 4), "unit": "Mphotons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's GLSL pipeline needs OpenGL, unavailable on this machine; this arm runs the CPU "
                "restatement of the reference's shaders (oracle/sppm_oracle.c) on the host cores",
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, local):
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    dev = local
    r, mesh, cfg, cam = make_renderer(dev, precision=1 if args.precision == "mixed" else 0)
    K, W = args.steps, args.warmup
    P = cfg.photon_width * cfg.photon_height
    npix = cfg.width * cfg.height
    clocks = ClockSampler(dev).__enter__()
    # warm-up passes (include at least one eye pass), then align to an eye-pass boundary so the
    # timed region holds exactly one eye pass per 10 passes
    r.run_passes(W)
    fi0 = r.frame_info()
    align = (10 - fi0.frames % 10) % 10
    if align:
        r.run_passes(align)
    r.synchronize()
    fi0 = r.frame_info()
    # device-timed region (CUDA events on the library's stream; each frame replays its CUDA
    # graph); the photon traversal kernel carries its own events for the roofline
    roof_stage = "photon_trace"
    r.time_stages([roof_stage])
    r.read_stage_times()
    barrier(world)
    t_wall = time.time()
    ms = r.time_passes(K)
    clocks.mark(t_wall, time.time())
    clocks.__exit__(None, None, None)
    roof_times = r.read_stage_times()[roof_stage]
    r.time_stages([])
    fi1 = r.frame_info()
    photons = fi1.photons_emitted - fi0.photons_emitted
    segments = (fi1.photon_segments + fi1.eye_segments) - (fi0.photon_segments + fi0.eye_segments)
    t = max_over_ranks(ms / 1000.0, world)
    photons_all = sum_over_ranks(photons, world)
    segs_all = sum_over_ranks(segments, world)
    value = photons_all / t / 1e6
    mrays = segs_all / t / 1e6
    launches = fi1.kernel_launches - fi0.kernel_launches

    # per-stage breakdown (every stage timed) over a further 10-pass cycle, outside the timed region
    r.enable_stage_timing(True)
    r.read_stage_times()
    r.run_passes(10)
    stages = r.read_stage_times()
    r.enable_stage_timing(False)

    # end to end through the public API with (page-locked) host buffers
    image = g.pinned_empty((cfg.height, cfg.width, 3), np.float32)
    E = max(10, min(K, 100))
    r.synchronize()
    fe0 = r.frame_info()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(E):
        r.set_camera(cam)
        r.run_passes(1)
        r.read_image(N.IMAGE_RADIANCE, out=image)
    te = time.perf_counter() - t0
    fe1 = r.frame_info()
    te = max_over_ranks(te, world)
    e2e_photons = sum_over_ranks(fe1.photons_emitted - fe0.photons_emitted, world)
    e2e = e2e_photons / te / 1e6

    # roofline of the photon kernel: algorithmic bytes per photon segment = 64 + 32 V + 36 T
    # (ray state in/out, 32-byte nodes, 36-byte triangles), V/T from the traversal counters
    peak, peak_kind = measured_peaks()
    kernel = "k_trace_photons4" if args.precision == "mixed" else "k_trace_photons"
    ph_ms, ph_n = roof_times
    roof = None
    if args.precision == "mixed":
        # the algorithmic bytes are those of the exact traversal of the same workload
        r32 = make_renderer(dev, precision=0)[0]
        r32.run_passes(W)
        cnt = traversal_counters(r32)
        r32.close()
    else:
        cnt = traversal_counters(r)
    if ph_n and cnt:
        seg_per_launch = cnt["photon_segments"] / cnt["passes"]
        bytes_per_launch = seg_per_launch * (64 + 32 * cnt["nodes_per_segment"] + 36 * cnt["tris_per_segment"])
        achieved = bytes_per_launch / (ph_ms / ph_n / 1000.0) / 1e9
        traffic = profile_traffic(kernel)
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": kernel,
                "peak_kind": peak_kind, "nodes_per_segment": round(cnt["nodes_per_segment"], 2),
                "tris_per_segment": round(cnt["tris_per_segment"], 2),
                "algorithmic_bytes_per_launch": round(bytes_per_launch)}

    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline and world == 1:
            res = cpu_baseline_run(max_seconds=args.cpu_seconds)
            cpu = {"value": round(res["photons"] / res["seconds"] / 1e6, 4), "unit": "Mphotons/s",
                   "cores": res["cores"], "kind": "port",
                   "sample": f"{res['frames']} passes from frame 0 of the same workload, {res['seconds']:.1f} s"}
        out = {
            "metric": "SPPM Mphotons/s + Mrays/s at fixed RMSE vs FP64 oracle, plain vs batched",
            "value": round(value, 3), "unit": "Mphotons/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": round(1000.0 * t / K, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(WORKLOAD, precision=args.precision, l2="working set > 129 MB L2 (no flush)",
                           parallelism=f"replicas x{world}"),
            "mrays_per_s": round(mrays, 3),
            "stage_ms_per_launch": {k: round(v[0] / v[1], 4) for k, v in stages.items() if v[1]},
            "gpu_launches": int(launches),
            "e2e": {"value": round(e2e, 3), "unit": "Mphotons/s", "h2d_bytes_per_step": 64,
                    "d2h_bytes_per_step": int(npix * 3 * 4), "steps": E},
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
        }
        print(json.dumps(out), flush=True)
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
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "mixed"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if args.impl == "reference" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
