"""Mixed-precision path (4-wide quantised BVH with FMA traversal, FP16 slot records, double-float
statistics) against the plain FP32 path and the FP64 oracle."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N

pytestmark = pytest.mark.gpu


def render(cfg, mesh, cam, passes):
    r = g.Renderer(cfg)
    r.upload_scene(mesh)
    r.set_camera(cam)
    r.run_passes(passes)
    r.synchronize()
    return r


def test_mixed_photon_hits_equal_fp32_on_the_same_rays(cornell_c1_mesh):
    """One frame from the same seeds: the same eye and photon rays; the quantised-box FMA traversal
    must report the same triangle as the exact traversal for (almost) every segment."""
    sc, mesh = cornell_c1_mesh
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 64, 64, sc.fov)
    base = dict(photon_width=256, photon_height=256, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.005)
    r32 = render(g.default_config(64, **base), mesh, cam, 1)
    rmx = render(g.default_config(64, precision=N.PRECISION_MIXED, **base), mesh, cam, 1)
    h32, hmx = r32.read_state("photon_hit"), rmx.read_state("photon_hit")
    same = h32[:, 0] == hmx[:, 0]
    assert same.mean() > 0.9995, f"{(~same).sum()} of {len(same)} photon hits differ"
    p32, pmx = r32.read_state("photon_position"), rmx.read_state("photon_position")
    both = same & (h32[:, 0] >= 0)
    rel = np.abs(p32[both, :3] - pmx[both, :3]).max() / np.abs(p32[both, :3]).max()
    assert rel < 1e-5, rel
    # the eye pass of the mixed path walks the 4-wide BVH too: the same visible triangle for
    # (almost) every pixel
    e32, emx = r32.read_state("hit_triangle"), rmx.read_state("hit_triangle")
    assert (e32 == emx).mean() > 0.999, f"{(e32 != emx).sum()} of {len(e32)} eye hits differ"


@pytest.mark.parametrize("scene", ["cornell", "materials", "environment"])
def test_mixed_image_error_vs_fp64_oracle_matches_fp32(cornell_c1_mesh, scene):
    """The Cornell box; every material class (glass, plastic, glossy); no light (photons from the
    environment)."""
    from oracle.binding import Oracle
    from glslppm_gb300 import scenes
    if scene == "cornell":
        sc, mesh = cornell_c1_mesh
    else:
        sc = scenes.materials_box(light=scene == "materials")
        mesh = sc.to_mesh()
    res, passes = 48, 120
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)
    base = dict(photon_width=128, photon_height=128, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.01)
    img32 = render(g.default_config(res, **base), mesh, cam, passes).read_image()
    imgmx = render(g.default_config(res, precision=N.PRECISION_MIXED, **base), mesh, cam, passes).read_image()
    o = Oracle(g.default_config(res, seed=12345, **base), mesh.scene(), cam, fp64=True)
    o.run_frames(passes)
    ref = o.read_image(0)
    mean = ref.mean()
    rmse32 = np.sqrt(((img32 - ref) ** 2).mean()) / mean
    rmsemx = np.sqrt(((imgmx - ref) ** 2).mean()) / mean
    assert np.isfinite(imgmx).all()
    assert rmsemx <= 1.1 * rmse32 + 0.01, (rmse32, rmsemx)
    # the two GPU paths start from the same random state: their images stay close
    assert np.sqrt(((imgmx - img32) ** 2).mean()) / mean < 0.5 * rmse32 + 0.02


def test_mixed_statistics_are_double_float(cornell_c1_mesh):
    """N, R^2 and tau arrive as doubles; kept as float pairs on the device, they carry more than
    single precision (N sums 0.7 * M over the passes)."""
    sc, mesh = cornell_c1_mesh
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)
    r = render(g.default_config(32, precision=N.PRECISION_MIXED, photon_width=64, photon_height=64,
                                radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.01), mesh, cam, 25)
    n, r2, tau = r.read_state("stats_n"), r.read_state("stats_r2"), r.read_state("stats_tau").reshape(-1, 3)
    assert n.dtype == np.float64 and r2.dtype == np.float64
    valid = r.read_state("hit_triangle") >= 0
    assert (n[valid] > 0).mean() > 0.5 and np.all(r2 > 0) and np.all(tau >= 0)
    r0 = 0.01 * np.sqrt(3.0)
    assert np.all(r2 <= r0 * r0 * (1 + 1e-6))
    wide = n[valid] != n[valid].astype(np.float32).astype(np.float64)
    assert wide.mean() > 0.1, wide.mean()
