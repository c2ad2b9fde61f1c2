"""Generates the golden fixtures of tests/golden (run on the development machine, where the
reference sources are present):

  cornell_metal_scene.npz  the reference's default scene (cornell_metal.obj, scale 0.01) as the
                           reference's own host code (mesh.cpp, bvh.cpp, camera.cpp, compiled from
                           its sources into oracle/_ref) loads it, plus its 512x512 camera;
  kat_rng.npz              the xorshift128 seed tables of a 512x512 run (RandomizeTextures) at
                           pixels {0, 1, 511, 512^2-1} and photons {0, 512^2-1}, with the first 64
                           GPURnd draws of each (oracle);
  kat_hash.npz             a seeded 64x64 photon set and its stochastic hashed grid (winner and
                           count per slot, oracle);
  kat_frames_cm32.npz      the oracle's state after 1, 10 and 23 frames of a 32x32 image with 32x32
                           photon slots on cornell_metal, with the camera used;
  cornell_box_scene.npz    the generated 7,948-triangle Cornell box of the 256x256 and 1024x1024
                           workloads (glslppm_gb300.scenes.cornell_box written as OBJ/MTL) as the
                           reference's own host code loads it and builds its BVH, with the
                           TCamera of its default view at 1024x1024: the scene of bench.py's CPU
                           reference arm, which must not use the product's loader or BVH builder.

usage: python tests/golden/make_golden.py [name ...]   (default: every fixture)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

from oracle.build import build_oracle, build_ref, reference_dir  # noqa: E402
from oracle.refdump import run_ref_host_dump  # noqa: E402

OUT = Path(__file__).resolve().parent


def save(name: str, **arrays) -> None:
    np.savez_compressed(OUT / name, **arrays)
    print("wrote", OUT / name, sum(np.asarray(a).nbytes for a in arrays.values()), "bytes (uncompressed)")


def scene_dict(d: dict) -> dict:
    out = {k: d[k] for k in ("positions", "normals", "texcoords", "material_ids", "light_triangles", "light_cdf",
                             "bbox_min", "bbox_max", "node_bounds", "node_triangle", "order_base", "order_miss")}
    out["light_area"] = np.float32(d["light_area"])
    out["mat_color"] = d["materials"]["color"]
    out["mat_eta"] = d["materials"]["eta"]
    out["mat_brdf"] = d["materials"]["brdf"]
    out["mat_glossiness"] = d["materials"]["glossiness"]
    for k in ("origin", "u", "v", "w"):
        out["cam_" + k] = np.asarray(d["camera"][k], dtype=np.float32)
    out["cam_distance"] = np.float32(d["camera"]["distance"])
    return out


def cornell_box_fixture() -> None:
    import tempfile

    from glslppm_gb300 import scenes
    sc = scenes.cornell_box()
    with tempfile.TemporaryDirectory() as td:
        obj = sc.write_obj(Path(td) / "cornell_box.obj")
        d = run_ref_host_dump(obj, 1.0, (sc.camera_origin, sc.camera_lookat, 1024, 1024, sc.fov))
    sd = scene_dict(d)
    sd["camera_origin"] = np.asarray(sc.camera_origin, np.float32)
    sd["camera_lookat"] = np.asarray(sc.camera_lookat, np.float32)
    sd["fov"] = np.float32(sc.fov)
    save("cornell_box_scene.npz", **sd)


def main(names: list[str]) -> None:
    build_oracle()
    build_ref(reference_dir())
    if names:
        for n in names:
            {"cornell_box_scene": cornell_box_fixture}[n]()
        return
    cornell_box_fixture()
    import glslppm_gb300 as g
    from oracle.binding import Oracle, gpurnd_sequence, hash_build
    from tests.golden.fixtures import camera_from, scene_arrays_from

    # 1. the reference's default scene, loaded by the reference's host code
    cm = run_ref_host_dump(reference_dir() / "cornell_metal.obj", 0.01, ((0, 0, 13), (0, 0, 0), 512, 512, 45))
    sd = scene_dict(cm)
    save("cornell_metal_scene.npz", **sd)
    arrays = scene_arrays_from(sd)
    scene = g.scene_from_arrays(arrays)

    # 2. seed tables and GPURnd sequences
    cfg = g.default_config(512)
    cam = camera_from(sd, 512, 512)
    o = Oracle(cfg, scene, cam)
    eye = o.read_state("eye_rng")
    pho = o.read_state("photon_rng")
    o.close()
    pix = np.array([0, 1, 511, 512 * 512 - 1])
    phs = np.array([0, 512 * 512 - 1])
    seeds = np.concatenate([eye[pix], pho[phs]])
    draws = np.stack([gpurnd_sequence(s, 64)[0] for s in seeds])
    finals = np.stack([gpurnd_sequence(s, 64)[1] for s in seeds])
    save("kat_rng.npz", eye_index=pix, photon_index=phs, seeds=seeds, draws=draws, final_state=finals)

    # 3. hashed grid of a seeded photon set
    rng = np.random.default_rng(20150317)
    pw = ph = 64
    pos = np.zeros((pw * ph, 4), np.float32)
    pos[:, :3] = rng.random((pw * ph, 3), dtype=np.float32)
    # cluster a quarter of the photons so that slots collide
    pos[: pw * ph // 4, :3] = 0.5 + 0.02 * rng.random((pw * ph // 4, 3), dtype=np.float32)
    flux = np.ones((pw * ph, 4), np.float32)
    flux[rng.random(pw * ph) < 0.2, 0] = -1.0  # invalid photons
    bbmin = np.array([-0.01, -0.02, -0.03], np.float32)
    G = np.float32(23.5)
    res = {}
    for hs in (4096, 1000):
        for flags in (0, 1):
            w, c = hash_build(pos, flux, pw, ph, hs, bbmin, float(G), flags)
            res[f"winner_{hs}_{flags}"] = w
            res[f"count_{hs}_{flags}"] = c
    save("kat_hash.npz", pos=pos, flux=flux, bbox_min=bbmin, grid_scale=G, photon_width=np.int32(pw),
         photon_height=np.int32(ph), **res)

    # 4. oracle state after K frames, 32x32, cornell_metal
    cfg = g.default_config(32)
    cam = camera_from(sd, 32, 32)
    cam.distance = np.float32(32.0) / (np.float32(2.0) * np.float32(np.tan(np.float32(22.5) * np.float32(3.141592 / 180.0))))
    o = Oracle(cfg, scene, cam)
    out = {"cam_distance_32": np.float32(cam.distance)}
    done = 0
    for k in (1, 10, 23):
        o.run_frames(k - done)
        done = k
        for kind in ("hit_triangle", "hit_position", "flux_radius", "emission_n", "photon_position", "photon_flux",
                     "photon_hit", "slot_winner", "slot_count"):
            out[f"{kind}_{k}"] = o.read_state(kind)
        out[f"radiance_{k}"] = o.read_image(0).astype(np.float32)
        fi = o.frame_info()
        out[f"photons_{k}"] = np.uint64(fi.photons_emitted)
    save("kat_frames_cm32.npz", **out)


if __name__ == "__main__":
    main(sys.argv[1:])
