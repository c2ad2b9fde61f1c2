"""Generates the converged reference of the 256x256 Cornell-box workload and the error-by-pass-count
calibration that serving targets and the bench's image-error figures use (test infrastructure; run
on the development machine, about 15 minutes on 8 cores):

  c1_converged_fp64.npz     the radiance image of the 256x256 workload's scene and camera (the
                            Cornell box of cornell_box_scene.npz, radius 0.5% of the scene diagonal,
                            alpha 0.7) rendered by the double-precision oracle to convergence: 4096
                            passes from each of two seeds that no test renders with (7 and 11),
                            averaged, each pass with 2^18 photon slots, an eye pass every pass and
                            the counting-sort grid estimator (every photon within the radius) --
                            the same limit image as the workload's own schedule (SPPM converges to
                            the pixel-filtered radiance for any photon count, eye-pass interval and
                            unbiased density estimator), reached with 2^31 photons and 4096 eye
                            samples; stored as float32, with the two runs' own relative difference;
  convergence_c1.json       the relative RMSE, against that reference, of the single-precision
                            image of the workload itself (2^16 photon slots, an eye pass every 10
                            passes, the default seed) after 16 ... 2048 passes, with the reference's
                            one-winner-per-slot estimator (the GPU's FP32 path renders these images
                            bit for bit) and with the grid estimator (the mixed path's
                            SPPM_FLAG_PHOTON_GRID, within 1e-4 of these images), the estimated error
                            of the reference itself, and for each a power-law fit err = a * ppp^-b
                            over photons per pixel.

usage: python tests/golden/make_converged_reference.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

from oracle.binding import Oracle  # noqa: E402
from oracle.structs import FLAG_PHOTON_GRID, RADIUS_DIAGONAL, camera_from_npz, default_config, scene_from_npz  # noqa: E402

OUT = Path(__file__).resolve().parent
RES = 256
REF_PASSES = 4096
REF_SEEDS = (7, 11)
REF_PHOTONS = 512  # photon slots per pass of the reference runs: 512 x 512
CURVE = (16, 32, 64, 128, 256, 512, 1024, 2048)


def c1_config(seed: int = 0, flags: int = 0):
    cfg = default_config(RES, radius_rule=RADIUS_DIAGONAL, radius_fraction=0.005, seed=seed)
    cfg.flags |= flags
    return cfg


def reference_config(seed: int):
    return default_config(RES, photon_width=REF_PHOTONS, photon_height=REF_PHOTONS, radius_rule=RADIUS_DIAGONAL,
                          radius_fraction=0.005, seed=seed, eye_pass_interval=1, flags=FLAG_PHOTON_GRID)


def c1_camera(d: dict):
    """TCamera::Set for 256x256: the fixture's 1024x1024 basis with distance H / (2 tan(22.5 deg))
    (stored with the reference, so that renders elsewhere use the same number)."""
    cam = camera_from_npz(d, RES, RES)
    cam.distance = np.float32(RES) / (np.float32(2.0) * np.float32(np.tan(np.float32(22.5) * np.float32(3.141592 / 180.0))))
    return cam


def rel_rmse(img: np.ndarray, ref: np.ndarray) -> float:
    return float(np.sqrt(np.mean((img.astype(np.float64) - ref) ** 2)) / np.sqrt(np.mean(ref.astype(np.float64) ** 2)))


def main() -> None:
    scene, d = scene_from_npz(OUT / "cornell_box_scene.npz")
    cam = c1_camera(d)
    runs = []
    for seed in REF_SEEDS:
        o = Oracle(reference_config(seed), scene, cam, fp64=True)
        o.run_frames(REF_PASSES)
        runs.append(o.read_image(0))
        o.close()
        print("reference run, seed", seed, "done", flush=True)
    ref = 0.5 * (runs[0] + runs[1])
    pair = rel_rmse(runs[0], runs[1])
    # two independent runs of error e each differ by sqrt(2) e; their mean has error e / sqrt(2)
    ref_err = pair / np.sqrt(2.0) / np.sqrt(2.0)
    np.savez_compressed(OUT / "c1_converged_fp64.npz", radiance=ref.astype(np.float32),
                        passes=np.int32(REF_PASSES), seeds=np.array(REF_SEEDS, np.int32),
                        runs_rel_rmse=np.float64(pair), cam_distance=np.float32(cam.distance))
    curves = {}
    for name, flags in (("winner", 0), ("grid", FLAG_PHOTON_GRID)):
        o = Oracle(c1_config(0, flags), scene, cam)
        curve = {}
        done = 0
        for k in CURVE:
            o.run_frames(k - done)
            done = k
            curve[k] = rel_rmse(o.read_image(0), ref)
            print(name, k, curve[k], flush=True)
        o.close()
        curves[name] = curve

    def fit(curve):
        # over photons per pixel (the workload emits 2^16 photons per pass over 2^16 pixels), on
        # the error with the reference's own error removed in quadrature
        ppp = np.array(CURVE, np.float64) * (2.0 ** 16) / (RES * RES)
        err = np.sqrt(np.maximum(np.array([curve[k] for k in CURVE]) ** 2 - ref_err ** 2, 1e-12))
        slope, icpt = np.polyfit(np.log(ppp), np.log(err), 1)
        return {"model": "rel_rmse = a * photons_per_pixel^-b (reference error removed in quadrature)",
                "a": float(np.exp(icpt)), "b": float(-slope)}

    out = {
        "workload": "Cornell box 256x256, 2^16 photon slots, radius 0.5% of the diagonal, alpha 0.7, eye pass "
                    "every 10 passes, seed 0",
        "reference": {"file": "c1_converged_fp64.npz", "passes": REF_PASSES, "seeds": list(REF_SEEDS),
                      "photon_slots_per_pass": REF_PHOTONS * REF_PHOTONS, "eye_pass_interval": 1,
                      "estimator": "counting-sort grid (every photon within the radius), FP64",
                      "photons": int(2 * REF_PASSES * REF_PHOTONS * REF_PHOTONS), "runs_rel_rmse": pair,
                      "estimated_rel_error": ref_err},
        "rel_rmse_by_passes": {str(k): v for k, v in curves["winner"].items()},
        "fit": fit(curves["winner"]),
        "grid_rel_rmse_by_passes": {str(k): v for k, v in curves["grid"].items()},
        "grid_fit": fit(curves["grid"]),
    }
    (OUT / "convergence_c1.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
