"""Batched SPPM (include/sppm_batch.h): many render jobs advanced by one launch per stage."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N
from .renderer import Mesh, SceneArrays, _check_image_buffer, _release_tickets, _state_array, scene_from_arrays


def _scene(scene):
    if isinstance(scene, Mesh):
        return scene.scene()
    if isinstance(scene, SceneArrays):
        return scene_from_arrays(scene)
    return scene


class Batch:
    """A set of resident render jobs on one GPU.  Job ids are small integers (slots)."""

    def __init__(self, precision: int = N.PRECISION_FP32, flags: int = 0, eye_pass_interval: int = 10,
                 max_jobs: int = 256, memory_budget: int = 0, device: int = 0):
        cfg = N.BatchConfig()
        N.lib.sppm_batch_config_defaults(C.byref(cfg))
        cfg.precision, cfg.flags, cfg.eye_pass_interval = precision, flags, eye_pass_interval
        cfg.max_jobs, cfg.memory_budget = max_jobs, memory_budget
        out = C.c_void_p()
        N.check(N.lib.sppm_batch_create(C.byref(cfg), device, C.byref(out)))
        self._h = out
        self.config = cfg
        self._sizes: dict[int, tuple[int, int]] = {}
        self._inflight: dict[int, np.ndarray] = {}  # host images of copies not yet waited for

    def job_bytes(self, config: N.Config, scene) -> int:
        n = C.c_uint64()
        N.check(N.lib.sppm_batch_job_bytes(self._h, C.byref(config), C.byref(_scene(scene)), C.byref(n)))
        return int(n.value)

    def add_job(self, config: N.Config, scene, camera: N.Camera) -> int:
        job = C.c_uint32()
        N.check(N.lib.sppm_batch_add_job(self._h, C.byref(config), C.byref(_scene(scene)), C.byref(camera),
                                         C.byref(job)))
        self._sizes[job.value] = (config.width, config.height)
        return int(job.value)

    def add_job_prepared(self, config: N.Config, prepared: "PreparedScene", camera: N.Camera,
                         state: "PreparedState | None" = None) -> int:
        """add_job with a scene (and optionally the random-state tables) prepared ahead of time."""
        job = C.c_uint32()
        N.check(N.lib.sppm_batch_add_job_prepared(self._h, C.byref(config), prepared._h,
                                                  state._h if state is not None else None, C.byref(camera),
                                                  C.byref(job)))
        self._sizes[job.value] = (config.width, config.height)
        return int(job.value)

    def remove_job(self, job: int) -> None:
        N.check(N.lib.sppm_batch_remove_job(self._h, job))
        self._sizes.pop(job, None)

    def reset_job(self, job: int) -> None:
        N.check(N.lib.sppm_batch_reset_job(self._h, job))

    def set_camera(self, job: int, camera: N.Camera) -> None:
        N.check(N.lib.sppm_batch_set_camera(self._h, job, C.byref(camera)))

    def set_cameras(self, jobs, cameras) -> None:
        """set_camera for every (job, camera) pair, the descriptor uploads queued as one launch."""
        jobs, cameras = list(jobs), list(cameras)
        if len(jobs) != len(cameras):
            raise ValueError(f"{len(jobs)} jobs but {len(cameras)} cameras")
        ids = (C.c_uint32 * len(jobs))(*jobs)
        cams = (N.Camera * len(cameras))(*cameras)
        N.check(N.lib.sppm_batch_set_cameras(self._h, len(jobs), ids, cams))

    def run_passes(self, n: int = 1) -> None:
        N.check(N.lib.sppm_batch_run_passes(self._h, n))

    def time_passes(self, n: int) -> float:
        ms = C.c_float()
        N.check(N.lib.sppm_batch_time_passes(self._h, n, C.byref(ms)))
        return float(ms.value)

    def set_tuning(self, tuning=None, **fields) -> None:
        """Launch shapes (sppm_tuning): an N.Tuning, or its fields by name (others 0 = default)."""
        t = tuning if tuning is not None else N.Tuning(**fields)
        N.check(N.lib.sppm_batch_set_tuning(self._h, C.byref(t)))

    def get_tuning(self) -> N.Tuning:
        t = N.Tuning()
        N.check(N.lib.sppm_batch_get_tuning(self._h, C.byref(t)))
        return t

    def autotune(self, cycles: int = 1) -> tuple[N.Tuning, float]:
        """Runs the next passes under candidate launch shapes and keeps the fastest; returns the
        shapes chosen and their device time per pass (ms)."""
        t, ms = N.Tuning(), C.c_float()
        N.check(N.lib.sppm_batch_autotune(self._h, cycles, C.byref(t), C.byref(ms)))
        return t, float(ms.value)

    def synchronize(self) -> None:
        N.check(N.lib.sppm_batch_synchronize(self._h))
        self._inflight.clear()

    def read_image(self, job: int, kind: int = N.IMAGE_RADIANCE, out: np.ndarray | None = None) -> np.ndarray:
        w, h = self._sizes[job]
        if out is None:
            out = np.empty((h, w, 3), dtype=np.float32)
        N.check(N.lib.sppm_batch_read_image(self._h, job, kind, out.ctypes.data, w * h * 3))
        return out

    def read_image_async(self, job: int, out: np.ndarray, kind: int = N.IMAGE_RADIANCE) -> int:
        """Renderer.read_image_async for one job; the ticket is the batch's."""
        w, h = self._sizes[job]
        _check_image_buffer(out, w, h)
        t = C.c_uint64()
        N.check(N.lib.sppm_batch_read_image_async(self._h, job, kind, out.ctypes.data, out.size, C.byref(t)))
        self._inflight[int(t.value)] = out
        return int(t.value)

    def image_wait(self, ticket: int) -> None:
        N.check(N.lib.sppm_batch_image_wait(self._h, ticket))
        _release_tickets(self._inflight, ticket)

    def image_done(self, ticket: int) -> bool:
        done = C.c_int()
        N.check(N.lib.sppm_batch_image_query(self._h, ticket, C.byref(done)))
        if done.value:
            _release_tickets(self._inflight, ticket)
        return bool(done.value)

    def read_state(self, job: int, kind: str) -> np.ndarray:
        k = N.STATE[kind]
        nbytes = int(N.lib.sppm_batch_state_bytes(self._h, job, k))
        if nbytes == 0:
            raise N.SppmError(N.ERR_ARG, f"state {kind} is not kept by job {job}")
        out = _state_array(kind, nbytes)
        N.check(N.lib.sppm_batch_read_state(self._h, job, k, out.ctypes.data, nbytes))
        return out

    def frame_info(self, job: int) -> N.FrameInfo:
        fi = N.FrameInfo()
        N.check(N.lib.sppm_batch_get_frame_info(self._h, job, C.byref(fi)))
        return fi

    def frame_infos(self, jobs) -> list:
        """frame_info of several jobs with one device-to-host copy."""
        jobs = list(jobs)
        ids = (C.c_uint32 * len(jobs))(*jobs)
        out = (N.FrameInfo * len(jobs))()
        N.check(N.lib.sppm_batch_get_frame_infos(self._h, ids, len(jobs), out))
        return list(out)

    def save_checkpoint(self, job: int) -> bytes:
        n = int(N.lib.sppm_batch_checkpoint_bytes(self._h, job))
        buf = C.create_string_buffer(n)
        N.check(N.lib.sppm_batch_save_checkpoint(self._h, job, buf, n))
        return buf.raw

    def load_checkpoint(self, job: int, data: bytes) -> None:
        N.check(N.lib.sppm_batch_load_checkpoint(self._h, job, data, len(data)))

    def info(self) -> N.BatchInfo:
        bi = N.BatchInfo()
        N.check(N.lib.sppm_batch_get_info(self._h, C.byref(bi)))
        return bi

    def time_stages(self, stages) -> None:
        mask = 0
        for s in stages:
            mask |= 1 << N.STAGES.index(s)
        N.check(N.lib.sppm_batch_set_stage_timing_mask(self._h, mask))

    def read_stage_times(self) -> dict:
        ms = (C.c_float * len(N.STAGES))()
        n = (C.c_uint32 * len(N.STAGES))()
        N.check(N.lib.sppm_batch_read_stage_times(self._h, ms, n))
        return {name: (float(ms[i]), int(n[i])) for i, name in enumerate(N.STAGES)}

    def traversal_counters(self, passes: int = 10) -> dict:
        """Mean BVH nodes visited and triangles tested per photon segment over every job."""
        jobs = list(self._sizes)
        f0 = [self.frame_info(j) for j in jobs]
        N.check(N.lib.sppm_batch_enable_traversal_counters(self._h, 1))
        try:
            self.run_passes(passes)
            self.synchronize()
        finally:
            N.check(N.lib.sppm_batch_enable_traversal_counters(self._h, 0))
        f1 = [self.frame_info(j) for j in jobs]
        segs = sum(b.counted_segments - a.counted_segments for a, b in zip(f0, f1))
        nodes = sum(b.counted_nodes - a.counted_nodes for a, b in zip(f0, f1))
        tris = sum(b.counted_triangles - a.counted_triangles for a, b in zip(f0, f1))
        return {"passes": passes, "photon_segments": segs, "nodes_per_segment": nodes / max(segs, 1),
                "tris_per_segment": tris / max(segs, 1)}

    @property
    def jobs(self) -> list[int]:
        return sorted(self._sizes)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            N.lib.sppm_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching render server (include/sppm_server.h): submit requests from any thread;
    a native thread admits them into a batch as slots and memory free up, runs passes of every
    resident job and retires finished ones."""

    def __init__(self, precision: int = N.PRECISION_FP32, flags: int = 0, eye_pass_interval: int = 10,
                 max_jobs: int = 256, memory_budget: int = 0, passes_per_step: int = 1, max_queue: int = 4096,
                 device: int = 0, tuning: dict | None = None):
        cfg = N.ServerConfig()
        N.lib.sppm_server_config_defaults(C.byref(cfg))
        cfg.batch.precision, cfg.batch.flags, cfg.batch.eye_pass_interval = precision, flags, eye_pass_interval
        cfg.batch.max_jobs, cfg.batch.memory_budget = max_jobs, memory_budget
        cfg.passes_per_step, cfg.max_queue = passes_per_step, max_queue
        if tuning:  # launch shapes of the server's batch, e.g. those Batch.autotune chose
            cfg.tuning = N.Tuning(**tuning)
        out = C.c_void_p()
        N.check(N.lib.sppm_server_create(C.byref(cfg), device, C.byref(out)))
        self._h = out
        self._sizes: dict[int, tuple[int, int]] = {}

    def submit(self, config: N.Config, scene, camera: N.Camera, target_passes: int) -> int:
        t = C.c_uint64()
        N.check(N.lib.sppm_server_submit(self._h, C.byref(config), C.byref(_scene(scene)), C.byref(camera),
                                         target_passes, C.byref(t)))
        self._sizes[t.value] = (config.width, config.height)
        return int(t.value)

    def poll(self, ticket: int) -> N.RequestInfo:
        info = N.RequestInfo()
        N.check(N.lib.sppm_server_poll(self._h, ticket, C.byref(info)))
        return info

    def wait(self, ticket: int, timeout: float = 60.0) -> N.RequestInfo:
        info = N.RequestInfo()
        N.check(N.lib.sppm_server_wait(self._h, ticket, timeout, C.byref(info)))
        return info

    def fetch_image(self, ticket: int) -> np.ndarray:
        w, h = self._sizes[ticket]
        out = np.empty((h, w, 3), dtype=np.float32)
        N.check(N.lib.sppm_server_fetch_image(self._h, ticket, out.ctypes.data, w * h * 3))
        del self._sizes[ticket]
        return out

    def stats(self) -> N.ServerStats:
        s = N.ServerStats()
        N.check(N.lib.sppm_server_get_stats(self._h, C.byref(s)))
        return s

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            N.lib.sppm_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PreparedScene:
    """sppm_scene_prepare: a scene's host-side upload work (traversal layout, 4-wide tree, leaf
    ranks) done on the calling thread; it owns its arrays and may be added to many jobs."""

    def __init__(self, scene):
        h = C.c_void_p()
        N.check(N.lib.sppm_scene_prepare(C.byref(_scene(scene)), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if self._h:
            N.lib.sppm_scene_prepared_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PreparedState:
    """sppm_state_prepare: a configuration's seeded random-state tables, made on the calling thread."""

    def __init__(self, config: N.Config):
        h = C.c_void_p()
        N.check(N.lib.sppm_state_prepare(C.byref(config), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if self._h:
            N.lib.sppm_state_prepared_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
