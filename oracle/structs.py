"""ctypes mirror of the plain-data structs of include/sppm.h that the CPU oracle takes (test
infrastructure: tests, smoke() and the CPU legs of bench.py).

The oracle is driven without the product library: ``oracle.binding.Oracle`` accepts these structs
(or the product's own ``glslppm_gb300.native`` structs, which have the same layout -- checked by
tests/test_abi.py), and ``scene_from_npz`` builds a scene from a committed fixture of the
reference's host code, so the reference arm of bench.py never loads ``libsppm.so``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

# sppm_radius_rule, sppm_seed_mode, flags (include/sppm.h)
RADIUS_FOOTPRINT, RADIUS_DIAGONAL = 0, 1
SEED_XORSHIFT, SEED_HASH = 0, 1
FLAG_GL_DEPTH_CLIP = 0x1
FLAG_PHOTON_GRID = 0x20


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


def default_config(resolution: int, **overrides) -> Config:
    """The reference's constants for a square image (glslppm.cpp:28-40, 488), the values
    sppm_config_defaults writes."""
    c = Config(width=resolution, height=resolution, photon_width=resolution, photon_height=resolution,
               hash_slots=0, max_path_length=10, eye_pass_interval=10, alpha=0.7, initial_footprint=2.5,
               radius_rule=RADIUS_FOOTPRINT, radius_fraction=0.005, precision=0, seed_mode=SEED_XORSHIFT, seed=0,
               flags=FLAG_GL_DEPTH_CLIP, focal_length=13.0, aperture=0.0)
    for k, v in overrides.items():
        if not hasattr(c, k):
            raise AttributeError(f"sppm_config has no field {k!r}")
        setattr(c, k, v)
    return c


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def scene_from_npz(path: str | Path) -> tuple[Scene, dict]:
    """An oracle Scene over the arrays of a scene fixture written by tests/golden/make_golden.py
    (the reference's own host code's TMesh + TBVH); returns (scene, fixture dict).  The struct keeps
    its arrays alive."""
    with np.load(path, allow_pickle=False) as z:
        d = {k: z[k] for k in z.files}
    arr = {
        "positions": np.ascontiguousarray(d["positions"], np.float32),
        "normals": np.ascontiguousarray(d["normals"], np.float32),
        "texcoords": np.ascontiguousarray(d["texcoords"], np.float32),
        "material_ids": np.ascontiguousarray(d["material_ids"], np.int32),
        "light_triangles": np.ascontiguousarray(d["light_triangles"], np.int32),
        "light_cdf": np.ascontiguousarray(d["light_cdf"], np.float32),
        "node_bounds": np.ascontiguousarray(d["node_bounds"], np.float32),
        "node_triangle": np.ascontiguousarray(d["node_triangle"], np.int32),
        "order_base": np.ascontiguousarray(d["order_base"], np.int32),
        "order_miss": np.ascontiguousarray(d["order_miss"], np.int32),
    }
    nm = len(d["mat_brdf"])
    mats = (Material * nm)()
    for i in range(nm):
        mats[i].color[:] = [float(x) for x in d["mat_color"][i]]
        mats[i].eta = float(d["mat_eta"][i])
        mats[i].brdf = int(d["mat_brdf"][i])
        mats[i].glossiness = float(d["mat_glossiness"][i])
    s = Scene()
    s.num_triangles = len(arr["material_ids"])
    s.positions = _ptr(arr["positions"], C.c_float)
    s.normals = _ptr(arr["normals"], C.c_float)
    s.texcoords = _ptr(arr["texcoords"], C.c_float)
    s.material_ids = _ptr(arr["material_ids"], C.c_int32)
    s.num_materials = nm
    s.materials = C.cast(mats, C.POINTER(Material))
    s.num_lights = len(arr["light_triangles"])
    s.light_triangles = _ptr(arr["light_triangles"], C.c_int32)
    s.light_cdf = _ptr(arr["light_cdf"], C.c_float)
    s.light_area = float(d["light_area"])
    s.bbox_min[:] = [float(x) for x in d["bbox_min"]]
    s.bbox_max[:] = [float(x) for x in d["bbox_max"]]
    s.num_nodes = len(arr["node_triangle"])
    s.node_bounds = _ptr(arr["node_bounds"], C.c_float)
    s.node_triangle = _ptr(arr["node_triangle"], C.c_int32)
    s.order_base = _ptr(arr["order_base"], C.c_int32)
    s.order_miss = _ptr(arr["order_miss"], C.c_int32)
    s.num_textures = 0
    s._keep = (arr, mats)
    return s, d


def camera_from_npz(d: dict, width: int, height: int) -> Camera:
    """The fixture's camera (TCamera after TCamera::Set, as the reference's camera.cpp computed it)."""
    cam = Camera()
    for k in ("origin", "u", "v", "w"):
        getattr(cam, k)[:] = [float(x) for x in d["cam_" + k]]
    cam.distance = float(d["cam_distance"])
    cam.width, cam.height = width, height
    return cam
