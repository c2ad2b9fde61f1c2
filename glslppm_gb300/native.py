"""ctypes binding of ``libsppm.so`` (the C ABI declared in ``include/sppm.h``).

Importing this module loads the in-tree native library and raises ``NativeLibraryMissing`` when it
has not been built -- there is no Python or CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libsppm.so"


class NativeLibraryMissing(ImportError):
    pass


class SppmError(RuntimeError):
    """A C ABI call returned a non-zero sppm_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"sppm status {status}: {message}")
        self.status = status


# sppm_status
OK, ERR_ARG, ERR_OOM, ERR_CUDA, ERR_WATCHDOG, ERR_STATE, ERR_IO, ERR_UNSUPPORTED, ERR_NO_DEVICE = range(9)
# enums
PRECISION_FP32, PRECISION_MIXED = 0, 1
RADIUS_FOOTPRINT, RADIUS_DIAGONAL = 0, 1
SEED_XORSHIFT, SEED_HASH = 0, 1
FLAG_GL_DEPTH_CLIP = 0x1
FLAG_FUSED_PHOTON = 0x2
FLAG_UNBINNED_RAYS = 0x4
FLAG_EAGER_LAUNCH = 0x8
FLAG_FP64_STATISTICS = 0x10
FLAG_PHOTON_GRID = 0x20
IMAGE_RADIANCE, IMAGE_DISPLAY = 0, 1
BVH_GPU_PLOC, BVH_GPU_LBVH = 0, 1
STAGES = ("frame_begin", "eye", "grid", "photon", "gather", "resolve", "photon_trace", "photon_store", "ray_bins",
          "photon_sort")

STATE = {
    "hit_position": 0, "hit_reflectance": 1, "hit_normal": 2, "eye_rng": 3, "hit_triangle": 4,
    "emission_n": 5, "flux_radius": 6, "photon_position": 7, "photon_flux": 8, "photon_direction": 9,
    "photon_rng": 10, "photon_hit": 11, "slot_winner": 12, "slot_count": 13, "hit_t": 14,
    "stats_n": 15, "stats_r2": 16, "stats_tau": 17,
}


class Config(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32),
        ("photon_width", C.c_uint32), ("photon_height", C.c_uint32),
        ("hash_slots", C.c_uint32), ("max_path_length", C.c_uint32), ("eye_pass_interval", C.c_uint32),
        ("alpha", C.c_float), ("initial_footprint", C.c_float),
        ("radius_rule", C.c_uint32), ("radius_fraction", C.c_float),
        ("precision", C.c_uint32), ("seed_mode", C.c_uint32), ("seed", C.c_uint32), ("flags", C.c_uint32),
        ("focal_length", C.c_float), ("aperture", C.c_float),
    ]


class Material(C.Structure):
    _fields_ = [("color", C.c_float * 3), ("eta", C.c_float), ("brdf", C.c_int32), ("glossiness", C.c_float)]


class Scene(C.Structure):
    _fields_ = [
        ("num_triangles", C.c_uint32),
        ("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
        ("texcoords", C.POINTER(C.c_float)), ("material_ids", C.POINTER(C.c_int32)),
        ("num_materials", C.c_uint32), ("materials", C.POINTER(Material)),
        ("num_lights", C.c_uint32), ("light_triangles", C.POINTER(C.c_int32)),
        ("light_cdf", C.POINTER(C.c_float)), ("light_area", C.c_float),
        ("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3),
        ("num_nodes", C.c_uint32), ("node_bounds", C.POINTER(C.c_float)),
        ("node_triangle", C.POINTER(C.c_int32)), ("order_base", C.POINTER(C.c_int32)),
        ("order_miss", C.POINTER(C.c_int32)),
        ("num_textures", C.c_uint32), ("textures", C.POINTER(C.c_uint8)),
        ("material_texture", C.POINTER(C.c_int32)),
    ]


class Camera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("u", C.c_float * 3), ("v", C.c_float * 3), ("w", C.c_float * 3),
                ("distance", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]


class FrameInfo(C.Structure):
    _fields_ = [
        ("frames", C.c_uint32), ("eye_samples", C.c_uint32), ("photons_emitted", C.c_uint64),
        ("num_photons_f32", C.c_float), ("initial_radius", C.c_float), ("grid_scale", C.c_float),
        ("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3), ("aa_offset", C.c_float * 2),
        ("photon_segments", C.c_uint64), ("eye_segments", C.c_uint64),
        ("counted_segments", C.c_uint64), ("counted_nodes", C.c_uint64), ("counted_triangles", C.c_uint64),
        ("coop_segments", C.c_uint64), ("kernel_launches", C.c_uint64),
    ]


class BatchConfig(C.Structure):
    _fields_ = [("precision", C.c_uint32), ("flags", C.c_uint32), ("eye_pass_interval", C.c_uint32),
                ("max_jobs", C.c_uint32), ("memory_budget", C.c_uint64)]


class BatchInfo(C.Structure):
    _fields_ = [("num_jobs", C.c_uint32), ("max_jobs", C.c_uint32), ("bytes_used", C.c_uint64),
                ("memory_budget", C.c_uint64), ("frames", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("photon_slots", C.c_uint64), ("pixels", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("trace_blocks_per_sm", C.c_uint32), ("trace_refill_steps", C.c_uint32), ("eye_block", C.c_uint32),
                ("store_block", C.c_uint32), ("gather_block", C.c_uint32), ("unbinned_rays", C.c_uint32),
                ("trace_tail_lanes", C.c_uint32), ("wide_bvh", C.c_uint32), ("photon_wave", C.c_uint32),
                ("grid_cell_split", C.c_uint32)]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("batch", BatchConfig), ("passes_per_step", C.c_uint32), ("max_queue", C.c_uint32),
                ("tuning", Tuning)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_uint32), ("status", C.c_int32), ("passes_done", C.c_uint32),
                ("target_passes", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("photons_emitted", C.c_uint64), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("failed", C.c_uint64), ("resident", C.c_uint32), ("queued", C.c_uint32),
                ("bytes_used", C.c_uint64), ("memory_budget", C.c_uint64), ("passes", C.c_uint64),
                ("photons", C.c_uint64), ("busy_seconds", C.c_double)]


REQUEST_QUEUED, REQUEST_RUNNING, REQUEST_DONE, REQUEST_FAILED = 0, 1, 2, 3


# every exported symbol of include/sppm.h, sppm_batch.h and sppm_server.h with its ctypes signature
P = C.c_void_p
SIGNATURES = {
    "sppm_config_defaults": (None, [C.POINTER(Config), C.c_uint32]),
    "sppm_camera_look_at": (None, [C.POINTER(Camera), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32,
                                   C.c_uint32, C.c_float]),
    "sppm_mesh_load_obj": (C.c_int, [C.c_char_p, C.POINTER(C.c_float), C.c_float, C.POINTER(P)]),
    "sppm_mesh_from_arrays": (C.c_int, [C.c_uint32, P, P, P, C.c_uint32, P, C.POINTER(P)]),
    "sppm_mesh_build_bvh": (C.c_int, [P]),
    "sppm_mesh_build_bvh_gpu": (C.c_int, [P, C.c_int]),
    "sppm_mesh_build_bvh_gpu_ex": (C.c_int, [P, C.c_int, C.c_int]),
    "sppm_mesh_get_scene": (C.c_int, [P, C.POINTER(Scene)]),
    "sppm_mesh_destroy": (None, [P]),
    "sppm_create": (C.c_int, [C.POINTER(Config), C.c_int, C.POINTER(P)]),
    "sppm_upload_scene": (C.c_int, [P, C.POINTER(Scene)]),
    "sppm_set_camera": (C.c_int, [P, C.POINTER(Camera)]),
    "sppm_reset": (C.c_int, [P]),
    "sppm_run_passes": (C.c_int, [P, C.c_uint32]),
    "sppm_synchronize": (C.c_int, [P]),
    "sppm_read_image": (C.c_int, [P, C.c_uint32, P, C.c_size_t]),
    "sppm_camera_upload_bytes": (C.c_size_t, []),
    "sppm_read_image_async": (C.c_int, [P, C.c_uint32, P, C.c_size_t, C.POINTER(C.c_uint64)]),
    "sppm_image_wait": (C.c_int, [P, C.c_uint64]),
    "sppm_image_query": (C.c_int, [P, C.c_uint64, C.POINTER(C.c_int)]),
    "sppm_read_state": (C.c_int, [P, C.c_uint32, P, C.c_size_t]),
    "sppm_state_bytes": (C.c_size_t, [P, C.c_uint32]),
    "sppm_checkpoint_bytes": (C.c_size_t, [P]),
    "sppm_save_checkpoint": (C.c_int, [P, P, C.c_size_t]),
    "sppm_load_checkpoint": (C.c_int, [P, P, C.c_size_t]),
    "sppm_get_frame_info": (C.c_int, [P, C.POINTER(FrameInfo)]),
    "sppm_enable_stage_timing": (C.c_int, [P, C.c_int]),
    "sppm_set_stage_timing_mask": (C.c_int, [P, C.c_uint32]),
    "sppm_enable_traversal_counters": (C.c_int, [P, C.c_int]),
    "sppm_read_stage_times": (C.c_int, [P, C.POINTER(C.c_float), C.POINTER(C.c_uint32)]),
    "sppm_time_passes": (C.c_int, [P, C.c_uint32, C.POINTER(C.c_float)]),
    "sppm_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "sppm_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "sppm_autotune": (C.c_int, [P, C.c_uint32, C.POINTER(Tuning), C.POINTER(C.c_float)]),
    "sppm_tune_hash_slots": (C.c_int, [C.POINTER(Config), C.POINTER(Scene), C.POINTER(Camera), C.c_int, C.c_uint32,
                                       C.POINTER(C.c_uint32), C.POINTER(C.c_float)]),
    "sppm_destroy": (None, [P]),
    "sppm_hash_build": (C.c_int, [P, P, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_float), C.c_float,
                                  C.c_uint32, P, P, P]),
    "sppm_reduce_texture": (C.c_int, [P, C.c_uint32, C.c_uint32, C.POINTER(C.c_float), P]),
    "sppm_reduce_texture_noalloc": (C.c_int, [P, C.c_uint32, C.c_uint32, C.POINTER(C.c_float), P]),
    "sppm_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "sppm_debug_fpmath": (C.c_int, [C.c_int, P, P, P, C.c_size_t]),
    "sppm_debug_trace": (C.c_int, [P, P, P, C.c_size_t, C.c_int, C.c_int, C.c_int, P, P]),
    "sppm_debug_photon_rays": (C.c_int, [P, P, P, P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "sppm_debug_photon_grid": (C.c_int, [P, P, C.c_size_t, P, C.c_size_t, C.POINTER(C.c_uint32)]),
    "sppm_debug_ray_bins": (C.c_int, [P, P, P, C.c_size_t, C.POINTER(C.c_uint32)]),
    "sppm_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(P)]),
    "sppm_write_image_file": (C.c_int, [C.c_char_p, P, C.c_uint32, C.c_uint32, C.c_uint32]),
    "sppm_host_free": (None, [P]),
    "sppm_device_count": (C.c_int, []),
    # include/sppm_batch.h
    "sppm_batch_config_defaults": (None, [C.POINTER(BatchConfig)]),
    "sppm_batch_create": (C.c_int, [C.POINTER(BatchConfig), C.c_int, C.POINTER(P)]),
    "sppm_batch_destroy": (None, [P]),
    "sppm_batch_job_bytes": (C.c_int, [P, C.POINTER(Config), C.POINTER(Scene), C.POINTER(C.c_uint64)]),
    "sppm_scene_prepare": (C.c_int, [C.POINTER(Scene), C.POINTER(P)]),
    "sppm_scene_prepared_destroy": (None, [P]),
    "sppm_batch_job_bytes_prepared": (C.c_int, [P, C.POINTER(Config), P, C.POINTER(C.c_uint64)]),
    "sppm_batch_add_job_prepared": (C.c_int, [P, C.POINTER(Config), P, P, C.POINTER(Camera), C.POINTER(C.c_uint32)]),
    "sppm_state_prepare": (C.c_int, [C.POINTER(Config), C.POINTER(P)]),
    "sppm_state_prepared_destroy": (None, [P]),
    "sppm_batch_add_job": (C.c_int, [P, C.POINTER(Config), C.POINTER(Scene), C.POINTER(Camera),
                                     C.POINTER(C.c_uint32)]),
    "sppm_batch_remove_job": (C.c_int, [P, C.c_uint32]),
    "sppm_batch_reset_job": (C.c_int, [P, C.c_uint32]),
    "sppm_batch_set_camera": (C.c_int, [P, C.c_uint32, C.POINTER(Camera)]),
    "sppm_batch_set_cameras": (C.c_int, [P, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(Camera)]),
    "sppm_batch_run_passes": (C.c_int, [P, C.c_uint32]),
    "sppm_batch_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "sppm_batch_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "sppm_batch_autotune": (C.c_int, [P, C.c_uint32, C.POINTER(Tuning), C.POINTER(C.c_float)]),
    "sppm_batch_time_passes": (C.c_int, [P, C.c_uint32, C.POINTER(C.c_float)]),
    "sppm_batch_synchronize": (C.c_int, [P]),
    "sppm_batch_read_image": (C.c_int, [P, C.c_uint32, C.c_uint32, P, C.c_size_t]),
    "sppm_batch_get_frame_infos": (C.c_int, [P, C.POINTER(C.c_uint32), C.c_uint32, P]),
    "sppm_batch_frame_record_bytes": (C.c_size_t, []),
    "sppm_batch_read_image_async": (C.c_int, [P, C.c_uint32, C.c_uint32, P, C.c_size_t, C.POINTER(C.c_uint64)]),
    "sppm_batch_image_wait": (C.c_int, [P, C.c_uint64]),
    "sppm_batch_image_query": (C.c_int, [P, C.c_uint64, C.POINTER(C.c_int)]),
    "sppm_batch_state_bytes": (C.c_size_t, [P, C.c_uint32, C.c_uint32]),
    "sppm_batch_read_state": (C.c_int, [P, C.c_uint32, C.c_uint32, P, C.c_size_t]),
    "sppm_batch_get_frame_info": (C.c_int, [P, C.c_uint32, C.POINTER(FrameInfo)]),
    "sppm_batch_get_info": (C.c_int, [P, C.POINTER(BatchInfo)]),
    "sppm_batch_checkpoint_bytes": (C.c_size_t, [P, C.c_uint32]),
    "sppm_batch_save_checkpoint": (C.c_int, [P, C.c_uint32, P, C.c_size_t]),
    "sppm_batch_load_checkpoint": (C.c_int, [P, C.c_uint32, P, C.c_size_t]),
    "sppm_batch_set_stage_timing_mask": (C.c_int, [P, C.c_uint32]),
    "sppm_batch_read_stage_times": (C.c_int, [P, P, P]),
    "sppm_batch_enable_traversal_counters": (C.c_int, [P, C.c_int]),
    # include/sppm_server.h
    "sppm_server_config_defaults": (None, [C.POINTER(ServerConfig)]),
    "sppm_server_create": (C.c_int, [C.POINTER(ServerConfig), C.c_int, C.POINTER(P)]),
    "sppm_server_destroy": (None, [P]),
    "sppm_server_submit": (C.c_int, [P, C.POINTER(Config), C.POINTER(Scene), C.POINTER(Camera), C.c_uint32,
                                     C.POINTER(C.c_uint64)]),
    "sppm_server_poll": (C.c_int, [P, C.c_uint64, C.POINTER(RequestInfo)]),
    "sppm_server_wait": (C.c_int, [P, C.c_uint64, C.c_double, C.POINTER(RequestInfo)]),
    "sppm_server_fetch_image": (C.c_int, [P, C.c_uint64, P, C.c_size_t]),
    "sppm_server_get_stats": (C.c_int, [P, C.POINTER(ServerStats)]),
    "sppm_abi_version": (C.c_uint32, []),
}


def _load() -> C.CDLL:
    path = Path(os.environ.get("SPPM_LIBRARY", LIB_PATH))
    if not path.exists():
        raise NativeLibraryMissing(
            f"{path} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(or `python glslppm_gb300/build.py`)")
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def last_error() -> str:
    buf = C.create_string_buffer(2048)
    lib.sppm_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != OK:
        raise SppmError(status, last_error())


def device_count() -> int:
    return int(lib.sppm_device_count())
