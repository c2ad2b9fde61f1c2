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


def primary_rays(cam, w, h):
    """A ray through the centre of every pixel from the camera's origin (TCamera's basis)."""
    o = np.array(cam.origin, np.float32)
    u, v, wv = (np.array(x, np.float32) for x in (cam.u, cam.v, cam.w))
    xs = (np.arange(w, dtype=np.float32) + 0.5) - w * 0.5
    ys = (np.arange(h, dtype=np.float32) + 0.5) - h * 0.5
    X, Y = np.meshgrid(xs, ys)
    d = X[..., None] * u + Y[..., None] * v + np.float32(cam.distance) * wv
    d = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32).reshape(-1, 3)
    return np.broadcast_to(o, d.shape).copy(), d


def classify(tri_e, t_e, tri_m, t_m):
    """Per ray: hit ids that differ must be ties (the same t, bit for bit) -- returns (mismatches,
    ties, rays that are neither)."""
    diff = tri_e != tri_m
    tie = diff & (t_e.view(np.uint32) == t_m.view(np.uint32))
    return int(diff.sum()), int(tie.sum()), np.nonzero(diff & ~tie)[0]


MIXED_CASES = {
    # the 1024x1024 workload with 2^20 photon slots (three passes: emission and two bounces)
    "cornell-1024": (lambda: __import__("bench").cornell_mesh(), 1024, 1024, 1024, 1024),
    # every material class of the reference's classifier (glass, plastic, glossy)
    "materials": (lambda: (lambda sc: (sc, sc.to_mesh()))(__import__("glslppm_gb300").scenes.materials_box()),
                  256, 256, 512, 512),
    # the batched workload's largest job (398k triangles: spheres and boxes in a Cornell box)
    "variant-398k": (lambda: (lambda j: (j.scene, j.scene.to_mesh()))(
        __import__("glslppm_gb300").scenes.cornell_variant(17)), 512, 512, 1024, 512),
}


@pytest.mark.parametrize("case", list(MIXED_CASES))
def test_mixed_hit_ids_are_exact_or_ties(case):
    """Every photon segment of three passes and every primary eye ray: the 4-wide quantised
    traversal must report the exact traversal's triangle and t -- at an equal t the triangle the
    exact walk meets first (the leaf ranks of its ordering).  A ray with another triangle fails the
    test, whether or not its t is the same.  The photon pass's own kernel (k_trace_photons4) must
    agree with the single-ray 4-wide walk on every one of its rays."""
    make, w, h, pw, ph = MIXED_CASES[case]
    sc, mesh = make()
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)
    cfg = g.default_config(w, height=h, photon_width=pw, photon_height=ph, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.005, precision=N.PRECISION_MIXED)
    r = g.Renderer(cfg)
    r.upload_scene(mesh)
    r.set_camera(cam)
    report = {}
    for frame in range(3):
        r.run_passes(1)
        org, dir, ph_idx = r.debug_photon_rays()
        assert len(org) > 0
        prod = r.read_state("photon_hit")[ph_idx, 0]
        tri_m, t_m = r.debug_trace(org, dir, photon=True, mode=3)
        assert np.array_equal(prod, tri_m), f"{case}: the photon kernel and the 4-wide walk disagree"
        tri_e, t_e = r.debug_trace(org, dir, photon=True, mode=0)
        n, ties, bad = classify(tri_e, t_e, tri_m, t_m)
        report[f"photon_frame{frame}"] = (len(org), n, ties)
        assert bad.size == 0, (f"{case} frame {frame}: {bad.size} of {len(org)} photon segments hit another "
                               f"triangle at another t; first: exact {tri_e[bad[:3]]} {t_e[bad[:3]]}, "
                               f"4-wide {tri_m[bad[:3]]} {t_m[bad[:3]]}")
        assert n == 0, f"{case} frame {frame}: {ties} ties broken unlike the exact walk"
        # the same triangle gives the same t (the triangle test is the exact path's)
        same = tri_e == tri_m
        assert np.array_equal(t_e[same].view(np.uint32), t_m[same].view(np.uint32))
    org, dir = primary_rays(cam, w, h)
    tri_e, t_e = r.debug_trace(org, dir, photon=False, cull=True, mode=0)
    tri_m, t_m = r.debug_trace(org, dir, photon=False, cull=True, mode=3)
    n, ties, bad = classify(tri_e, t_e, tri_m, t_m)
    report["eye"] = (len(org), n, ties)
    assert bad.size == 0, f"{case}: {bad.size} eye rays hit another triangle at another t"
    assert n == 0, f"{case}: {ties} eye-ray ties broken unlike the exact walk"
    print(case, "rays, mismatches, ties:", report)


def rel_rmse(img, ref):
    return float(np.sqrt(np.mean((img.astype(np.float64) - ref) ** 2)) / np.sqrt(np.mean(ref ** 2)))


def fp64_reference(cfg, scene, cam, passes):
    """The double-precision oracle with the same seed and random sequence (its GPURnd and cell
    hash are the single-precision ones): what a GPU image differs from is precision, not noise."""
    from oracle.binding import Oracle
    o = Oracle(cfg, scene, cam, fp64=True)
    o.run_frames(passes)
    ref = o.read_image(0)
    o.close()
    return ref


@pytest.mark.parametrize("scene", ["cornell-256", "materials", "environment"])
def test_mixed_image_error_vs_fp64_oracle_within_one_percent(cornell_c1_mesh, scene):
    """The 256x256 workload in full (2^16 photons, 64 passes); every material class; no light
    (photons from the environment): the mixed path's radiance image, and the FP32 path's, within 1%
    relative RMSE of the same-sequence FP64 oracle, and within 1% of each other."""
    from glslppm_gb300 import scenes
    if scene == "cornell-256":
        sc, mesh = cornell_c1_mesh
        res, pw, passes = 256, 256, 64
    else:
        sc = scenes.materials_box(light=scene == "materials")
        mesh = sc.to_mesh()
        res, pw, passes = 64, 128, 64
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)
    base = dict(photon_width=pw, photon_height=pw, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.005)
    img32 = render(g.default_config(res, **base), mesh, cam, passes).read_image()
    imgmx = render(g.default_config(res, precision=N.PRECISION_MIXED, **base), mesh, cam, passes).read_image()
    ref = fp64_reference(g.default_config(res, **base), mesh.scene(), cam, passes)
    e32, emx, e3m = rel_rmse(img32, ref), rel_rmse(imgmx, ref), rel_rmse(imgmx, img32.astype(np.float64))
    print(f"{scene}: relative RMSE vs FP64 oracle: FP32 {e32:.2e}, mixed {emx:.2e}; mixed vs FP32 {e3m:.2e}")
    assert np.isfinite(imgmx).all()
    assert e32 <= 0.01 and emx <= 0.01 and e3m <= 0.01, (e32, emx, e3m)


def test_double_float_statistics_hold_like_fp64_over_2000_passes(cornell_c1_mesh):
    """2000 passes at 64x64: the mixed path with double-float N, R^2, tau and the same path with
    IEEE double statistics (SPPM_FLAG_FP64_STATISTICS) stay together -- statistics within 1e-4
    relative for 99% of the pixels, images within 0.1% -- and both stay within 1% of the
    same-sequence FP64 oracle (progressive.fs:131-137 iterated 2000 times)."""
    sc, mesh = cornell_c1_mesh
    res, passes = 64, 2000
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)
    base = dict(photon_width=64, photon_height=64, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.005)
    rdf = render(g.default_config(res, precision=N.PRECISION_MIXED, **base), mesh, cam, passes)
    r64 = render(g.default_config(res, precision=N.PRECISION_MIXED, flags=N.FLAG_GL_DEPTH_CLIP | N.FLAG_FP64_STATISTICS,
                                  **base), mesh, cam, passes)
    valid = rdf.read_state("hit_triangle") >= 0
    for kind in ("stats_n", "stats_r2", "stats_tau"):
        a = rdf.read_state(kind).reshape(len(valid), -1)[valid]
        b = r64.read_state(kind).reshape(len(valid), -1)[valid]
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
        print(f"{kind}: median {np.median(rel):.2e}, p99 {np.percentile(rel, 99):.2e}, max {rel.max():.2e}")
        assert np.percentile(rel, 99) < 1e-4, kind
    idf, i64 = rdf.read_image(), r64.read_image()
    ref = fp64_reference(g.default_config(res, **base), mesh.scene(), cam, passes)
    e_df, e_64, e_pair = rel_rmse(idf, ref), rel_rmse(i64, ref), rel_rmse(idf, i64.astype(np.float64))
    print(f"2000 passes: double-float vs FP64 statistics {e_pair:.2e}; vs FP64 oracle: df {e_df:.2e}, fp64 {e_64:.2e}")
    assert e_pair <= 1e-3 and e_df <= 0.01 and e_64 <= 0.01, (e_pair, e_df, e_64)


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
