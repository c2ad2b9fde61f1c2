"""The oracle's counting-sort grid estimator (SPPM_FLAG_PHOTON_GRID), on the CPU: the photons it
gathers are exactly the stored photons within the radius of each hit point and facing it (a brute
force over all photons), and its single-precision restatement of the GPU's quantised records stays
within the precision budget of its double-precision form."""
from pathlib import Path

import numpy as np

from oracle.binding import Oracle
from oracle.structs import FLAG_PHOTON_GRID, RADIUS_DIAGONAL, camera_from_npz, default_config, scene_from_npz

GOLDEN = Path(__file__).resolve().parent / "golden"


def cornell(res):
    scene, d = scene_from_npz(GOLDEN / "cornell_box_scene.npz")
    return scene, camera_from_npz(d, res, res)


def cfg(res, pw, **kw):
    return default_config(res, photon_width=pw, photon_height=pw, radius_rule=RADIUS_DIAGONAL,
                          radius_fraction=0.01, flags=FLAG_PHOTON_GRID, **kw)


def test_grid_gathers_every_photon_within_the_radius():
    """One pass (every pixel at the initial radius), double precision: the photon count each
    pixel gathers (N = 0.7 M) equals a brute-force count over all stored photons of those inside
    the radius and facing the hit point."""
    res, pw = 48, 96
    scene, cam = cornell(res)
    o = Oracle(cfg(res, pw), scene, cam, fp64=True)
    o.run_frames(1)
    r0 = float(o.frame_info().initial_radius)
    qpos = o.read_state("hit_position")[:, :3].astype(np.float64)
    qnrm = o.read_state("hit_normal")[:, :3].astype(np.float64)
    tri = o.read_state("hit_triangle")
    m = np.rint(o.read_state("emission_n")[:, 3].astype(np.float64) / 0.7)
    ppos = o.read_state("photon_position")[:, :3].astype(np.float64)
    pflux = o.read_state("photon_flux")[:, :3]
    pdir = o.read_state("photon_direction")[:, :3].astype(np.float64)
    o.close()
    stored = pflux[:, 0] >= 0
    ppos, pdir = ppos[stored], pdir[stored]
    assert stored.sum() > 1000
    want = np.zeros(len(qpos))
    for i in np.nonzero(tri >= 0)[0]:
        d = np.linalg.norm(ppos - qpos[i], axis=1)
        face = (pdir @ -qnrm[i]) > 0
        want[i] = np.count_nonzero((d < r0) & face)
    valid = tri >= 0
    # positions are read back rounded to float32: a photon within ~1e-6 of the radius may flip
    diff = np.abs(m - want)[valid]
    assert (want[valid] > 0).mean() > 0.3
    assert diff.max() <= 1 and (diff > 0).mean() < 2e-3, (diff.max(), (diff > 0).mean())


def test_single_precision_grid_within_precision_budget_of_fp64():
    """Twelve passes (two eye passes) at 64x64 with 2^14 photon slots: the single-precision grid
    estimator (21-bit positions, FP16 flux, 8-bit directions, FP32 statistics) against the
    double-precision one (unquantised, FP64), same seed and random sequence: within 1% relative
    RMSE, and the two gather the same photon totals within 0.5%."""
    res, pw = 64, 128
    scene, cam = cornell(res)
    out = {}
    for fp64 in (False, True):
        o = Oracle(cfg(res, pw), scene, cam, fp64=fp64)
        o.run_frames(12)
        out[fp64] = (o.read_image(0).astype(np.float64), o.read_state("emission_n")[:, 3].astype(np.float64))
        o.close()
    (i32, n32), (i64, n64) = out[False], out[True]
    e = float(np.sqrt(np.mean((i32 - i64) ** 2)) / np.sqrt(np.mean(i64 ** 2)))
    assert e < 0.01, e
    assert abs(n32.sum() / n64.sum() - 1.0) < 5e-3
