"""Exact traversal on single rays: one ray per thread, one ray per warp, and the oracle's
raytrace() agree bit for bit -- on generic rays and on rays with zero direction components, whose
slab tests produce NaN and which the photon pass hands to the warp-cooperative walk."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N
from oracle.binding import Oracle

pytestmark = pytest.mark.gpu

AXES = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], dtype=np.float32)


def degenerate_rays(rng, lo, hi, n_each=48):
    """Origins on the six bounding planes of the scene and inside it, directions along the axes
    (also with -0.0 components) or with exactly one zero component."""
    orgs, dirs = [], []
    for axis in range(3):
        for plane in (lo[axis], hi[axis]):
            o = rng.uniform(lo, hi, size=(n_each, 3)).astype(np.float32)
            o[:, axis] = plane
            for d in AXES:
                orgs.append(o)
                dirs.append(np.repeat(d[None], n_each, 0))
            d = rng.normal(size=(n_each, 3)).astype(np.float32)
            d[:, (axis + 1) % 3] = 0.0
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            orgs.append(o)
            dirs.append(d.astype(np.float32))
    o = rng.uniform(lo, hi, size=(n_each, 3)).astype(np.float32)
    orgs.append(o)
    dirs.append(np.repeat(np.array([[-0.0, -1.0, -0.0]], dtype=np.float32), n_each, 0))
    return np.concatenate(orgs), np.concatenate(dirs)


@pytest.fixture(scope="module")
def traced(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(16, photon_width=16, photon_height=16)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 16, 16, sc.fov)
    r = g.Renderer(cfg)
    r.upload_scene(mesh)
    o = Oracle(cfg, mesh.scene(), cam)
    pos = mesh.arrays().positions.reshape(-1, 3)
    lo, hi = pos.min(0), pos.max(0)
    return r, o, lo, hi


@pytest.mark.parametrize("photon,cull", [(True, False), (False, True), (False, False)])
def test_thread_warp_and_oracle_agree_on_generic_rays(traced, photon, cull):
    r, o, lo, hi = traced
    rng = np.random.default_rng(5 + photon * 2 + cull)
    org = rng.uniform(lo + 0.01, hi - 0.01, size=(4096, 3)).astype(np.float32)
    d = rng.normal(size=(4096, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tri0, t0 = r.debug_trace(org, d, photon, cull, mode=0)
    trio, to = o.trace(org, d, photon, cull)
    assert (tri0 >= 0).mean() > 0.5
    np.testing.assert_array_equal(tri0, trio)
    np.testing.assert_array_equal(t0.view(np.uint32), to.view(np.uint32))
    for mode in (1, 2):
        trim, tm = r.debug_trace(org, d, photon, cull, mode=mode)
        np.testing.assert_array_equal(trim, trio, err_msg=f"mode {mode}")
        np.testing.assert_array_equal(tm.view(np.uint32), to.view(np.uint32), err_msg=f"mode {mode}")


@pytest.mark.parametrize("photon", [True, False])
def test_thread_warp_and_oracle_agree_on_zero_direction_components(traced, photon):
    r, o, lo, hi = traced
    org, d = degenerate_rays(np.random.default_rng(11), lo, hi)
    trio, to = o.trace(org, d, photon, False)
    for mode in (2, 1, 0):
        trim, tm = r.debug_trace(org, d, photon, False, mode=mode)
        np.testing.assert_array_equal(trim, trio, err_msg=f"mode {mode}")
        np.testing.assert_array_equal(tm.view(np.uint32), to.view(np.uint32), err_msg=f"mode {mode}")


def test_block_walk_on_a_large_scene(cornell_c1_mesh):
    """The block-per-ray walk over a 100k-triangle scene (windows of 1024 nodes, jumps between
    windows, several closest-hit updates per window) equals the thread-per-ray walk."""
    from glslppm_gb300 import scenes
    sc = scenes.cornell_variant(5, min_tris=90_000, max_tris=110_000).scene
    r = g.Renderer(g.default_config(16, photon_width=16, photon_height=16))
    r.upload_scene(sc.to_mesh())
    pos = sc.positions.reshape(-1, 3)
    org, d = degenerate_rays(np.random.default_rng(4), pos.min(0), pos.max(0), n_each=8)
    rng = np.random.default_rng(6)
    og = rng.uniform(0.05, 0.95, size=(512, 3)).astype(np.float32)
    dg = rng.normal(size=(512, 3))
    dg = (dg / np.linalg.norm(dg, axis=1, keepdims=True)).astype(np.float32)
    org, d = np.concatenate([org, og]), np.concatenate([d, dg])
    for photon in (True, False):
        tri0, t0 = r.debug_trace(org, d, photon, False, mode=0)
        tri2, t2 = r.debug_trace(org, d, photon, False, mode=2)
        np.testing.assert_array_equal(tri2, tri0)
        np.testing.assert_array_equal(t2.view(np.uint32), t0.view(np.uint32))


def test_photon_pass_with_warp_traced_segments_matches_fused_kernel(cornell_c1_mesh):
    """2^20 photons for 120 frames: some photons leave the light exactly straight down (a zero
    direction component), which the wavefront pass traces one per warp; the single-kernel pass
    traces every segment one per thread.  Both states are the same word for word."""
    sc, mesh = cornell_c1_mesh
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 64, 64, sc.fov)
    out = []
    for fused in (False, True):
        cfg = g.default_config(64, photon_width=1024, photon_height=1024, radius_rule=N.RADIUS_DIAGONAL,
                               radius_fraction=0.005)
        if fused:
            cfg.flags |= N.FLAG_FUSED_PHOTON
        r = g.Renderer(cfg)
        r.upload_scene(mesh)
        r.set_camera(cam)
        r.run_passes(120)
        r.synchronize()
        out.append((r.frame_info(), {k: r.read_state(k) for k in
                                     ("photon_position", "photon_flux", "photon_direction", "photon_rng",
                                      "photon_hit", "slot_winner", "slot_count", "flux_radius", "emission_n")}))
    (fw, sw), (ff, sf) = out
    assert fw.coop_segments > 0, "no photon segment with a zero direction component in this run"
    assert ff.coop_segments == 0
    assert fw.photon_segments == ff.photon_segments
    for k in sw:
        np.testing.assert_array_equal(np.ascontiguousarray(sw[k]).view(np.uint8),
                                      np.ascontiguousarray(sf[k]).view(np.uint8), err_msg=k)
