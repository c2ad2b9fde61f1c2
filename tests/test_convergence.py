"""The converged FP64 reference of the 256x256 workload and its error calibration
(tests/golden/make_converged_reference.py): the committed figures are consistent, and the GPU's
FP32 path, which renders the oracle's single-precision images bit for bit, reproduces them."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def calibration():
    return json.loads((GOLDEN / "convergence_c1.json").read_text())


def rel_rmse(img, ref):
    a = np.asarray(img, np.float64)
    return float(np.sqrt(np.mean((a - ref) ** 2)) / np.sqrt(np.mean(ref ** 2)))


def test_converged_reference_and_calibration_are_consistent():
    cal = calibration()
    with np.load(GOLDEN / "c1_converged_fp64.npz") as z:
        ref = z["radiance"]
        assert ref.shape == (256, 256, 3) and np.isfinite(ref).all() and ref.min() >= 0
        assert int(z["passes"]) == cal["reference"]["passes"] == 4096
    # two independent 4096-pass renders (2^31 photons, 4096 eye samples each) agree to ~0.5%: the
    # reference's own error ~0.3%
    assert cal["reference"]["estimated_rel_error"] < 0.005
    for curve, fit in (("rel_rmse_by_passes", "fit"), ("grid_rel_rmse_by_passes", "grid_fit")):
        errs = {int(k): v for k, v in cal[curve].items()}
        assert errs[2048] < errs[512] < errs[128] < errs[16]
        assert 0.3 < cal[fit]["b"] < 0.8  # about 1/sqrt(photons per pixel)
    # the grid estimator (every photon within the radius) is never noisier than one winner per slot
    assert all(cal["grid_rel_rmse_by_passes"][k] <= cal["rel_rmse_by_passes"][k] for k in cal["rel_rmse_by_passes"])


def test_serving_targets_from_the_calibration():
    import bench
    # the 256x256 workload itself (one photon per pixel per pass): 2% takes ~2070 passes
    p2 = bench.passes_for_target(0.02, 256 * 256, 1 << 16)
    assert 1000 < p2 < 4000
    # a quarter of the photons per pass takes four times the passes
    assert bench.passes_for_target(0.02, 256 * 256, 1 << 14) == pytest.approx(4 * p2, rel=0.01)
    assert bench.passes_for_target(0.10, 256 * 256, 1 << 16) < p2
    # more photons per pixel per pass than the calibration workload: still its pass count
    assert bench.passes_for_target(0.02, 128 * 128, 1 << 19) == p2
    # the grid estimator needs fewer passes for the same target
    assert bench.passes_for_target(0.02, 256 * 256, 1 << 16, fit="grid_fit") < p2


@pytest.mark.gpu
def test_gpu_reproduces_the_calibration():
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    from tests.golden.fixtures import c1_camera_and_scene
    cal = calibration()
    with np.load(GOLDEN / "c1_converged_fp64.npz") as z:
        ref = z["radiance"].astype(np.float64)
    scene, cam = c1_camera_and_scene()
    r = g.Renderer(g.default_config(256, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.005))
    r.upload_scene(scene)
    r.set_camera(cam)
    done = 0
    for k in (64, 256):
        r.run_passes(k - done)
        done = k
        err = rel_rmse(r.read_image(), ref)
        assert err == pytest.approx(cal["rel_rmse_by_passes"][str(k)], rel=1e-6), (k, err)


@pytest.mark.gpu
def test_gpu_grid_reproduces_the_grid_calibration():
    """The mixed path with the counting-sort grid, whose images are within 1e-4 of the
    single-precision oracle's grid estimator's, reaches the grid curve's errors to 1e-3 relative."""
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    from tests.golden.fixtures import c1_camera_and_scene
    cal = calibration()
    with np.load(GOLDEN / "c1_converged_fp64.npz") as z:
        ref = z["radiance"].astype(np.float64)
    scene, cam = c1_camera_and_scene()
    cfg = g.default_config(256, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.005, precision=N.PRECISION_MIXED)
    cfg.flags |= N.FLAG_PHOTON_GRID
    r = g.Renderer(cfg)
    r.upload_scene(scene)
    r.set_camera(cam)
    done = 0
    for k in (64, 256):
        r.run_passes(k - done)
        done = k
        err = rel_rmse(r.read_image(), ref)
        assert err == pytest.approx(cal["grid_rel_rmse_by_passes"][str(k)], rel=1e-3), (k, err)
