"""Loaders of the committed golden fixtures (made by tests/golden/make_golden.py)."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent


def load_npz(name: str) -> dict:
    with np.load(GOLDEN / name, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def scene_arrays_from(d: dict):
    from glslppm_gb300.renderer import MATERIAL_DTYPE, SceneArrays
    mats = np.zeros(len(d["mat_brdf"]), dtype=MATERIAL_DTYPE)
    mats["color"] = d["mat_color"]
    mats["eta"] = d["mat_eta"]
    mats["brdf"] = d["mat_brdf"]
    mats["glossiness"] = d["mat_glossiness"]
    return SceneArrays(
        positions=d["positions"], normals=d["normals"], texcoords=d["texcoords"], material_ids=d["material_ids"],
        materials=mats, light_triangles=d["light_triangles"], light_cdf=d["light_cdf"],
        light_area=float(d["light_area"]), bbox_min=d["bbox_min"], bbox_max=d["bbox_max"],
        node_bounds=d["node_bounds"], node_triangle=d["node_triangle"], order_base=d["order_base"],
        order_miss=d["order_miss"])


def camera_from(d: dict, width: int, height: int):
    from glslppm_gb300.native import Camera
    cam = Camera()
    for k in ("origin", "u", "v", "w"):
        getattr(cam, k)[:] = [float(x) for x in d["cam_" + k]]
    cam.distance = float(d["cam_distance"])
    cam.width, cam.height = width, height
    return cam


def load_cornell_metal():
    """(scene arrays, raw dict) of the reference's cornell_metal.obj as its host code loads it."""
    d = load_npz("cornell_metal_scene.npz")
    return scene_arrays_from(d), d


def c1_camera_and_scene():
    """The 256x256 workload's scene (the Cornell box as the reference's host code loads it) and
    camera, exactly as tests/golden/make_converged_reference.py rendered its converged reference."""
    import glslppm_gb300 as g
    d = load_npz("cornell_box_scene.npz")
    scene = g.scene_from_arrays(scene_arrays_from(d))
    cam = camera_from(d, 256, 256)
    cam.distance = float(load_npz("c1_converged_fp64.npz")["cam_distance"])
    return scene, cam
