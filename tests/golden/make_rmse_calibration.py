"""Relative RMSE against the FP64 oracle as a function of the pass count (writes
rmse_calibration.json beside this file).

Scene: the generated Cornell box at 64x64, radius 0.5% of the scene diagonal, alpha 0.7, hashed
seeding.  Reference: the FP64 oracle with another seed after 2^26 photons (16384 passes of 2^12).
Test: the FP32 oracle -- bit-identical to the GPU FP32 path -- at 16, 32, ..., 8192 passes of 2^12
photons.  relative RMSE = sqrt(mean((image - reference)^2)) / mean(reference), linear radiance.

    python tests/golden/make_rmse_calibration.py
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

import glslppm_gb300 as g  # noqa: E402
from glslppm_gb300 import native as N, scenes  # noqa: E402
from oracle.binding import Oracle  # noqa: E402


def main():
    sc = scenes.cornell_box()
    mesh = sc.to_mesh()
    res, side = 64, 64
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)

    def cfg(seed):
        return g.default_config(res, photon_width=side, photon_height=side, radius_rule=N.RADIUS_DIAGONAL,
                                radius_fraction=0.005, seed=seed, seed_mode=N.SEED_HASH)

    n_ref = (1 << 26) // (side * side)
    ref = Oracle(cfg(999), mesh.scene(), cam, fp64=True)
    ref.run_frames(n_ref)
    R = ref.read_image(0)
    o = Oracle(cfg(1), mesh.scene(), cam)
    curve, done, n = [], 0, 16
    while n <= n_ref // 2:
        o.run_frames(n - done)
        done = n
        img = o.read_image(0)
        curve.append([n, round(float(np.sqrt(((img - R) ** 2).mean()) / R.mean()), 5)])
        n *= 2
    out = {"scene": "cornell_box", "image": [res, res], "photons_per_pass": side * side,
           "radius": "0.5% of diagonal", "reference": {"precision": "fp64", "seed": 999, "passes": n_ref},
           "test": {"precision": "fp32 (= GPU FP32 path)", "seed": 1},
           "relative_rmse_by_passes": curve}
    (HERE / "rmse_calibration.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(curve))


if __name__ == "__main__":
    main()
