"""Checkpoint / resume: a render saved after k passes and loaded into a fresh context (or moved
between a batch and a single-job context) continues bit for bit like the uninterrupted render."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N, scenes

pytestmark = pytest.mark.gpu

KINDS = ["hit_position", "hit_triangle", "emission_n", "flux_radius", "photon_position", "photon_flux",
         "photon_rng", "photon_hit", "eye_rng"]


def setup(cfg, mesh, cam):
    r = g.Renderer(cfg)
    r.upload_scene(mesh)
    r.set_camera(cam)
    return r


def same(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("precision", [N.PRECISION_FP32, N.PRECISION_MIXED])
def test_resume_in_a_fresh_context(cornell_c1_mesh, precision):
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(32, photon_width=48, photon_height=40, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.01,
                           precision=precision)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)
    a = setup(cfg, mesh, cam)
    a.run_passes(13)  # mid eye-pass cycle
    ck = a.save_checkpoint()
    a.run_passes(9)
    b = setup(cfg, mesh, cam)
    b.run_passes(2)  # some unrelated progress, overwritten by the checkpoint
    b.load_checkpoint(ck)
    b.run_passes(9)
    kinds = KINDS + (["stats_n", "stats_r2", "stats_tau"] if precision == N.PRECISION_MIXED else [])
    for k in kinds:
        assert same(a.read_state(k), b.read_state(k)), k
    assert same(a.read_image(), b.read_image())
    fa, fb = a.frame_info(), b.frame_info()
    assert fa.frames == fb.frames == 22 and fa.photons_emitted == fb.photons_emitted
    assert fa.eye_samples == fb.eye_samples == 3


def test_move_a_job_from_a_batch_to_a_context(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(24, photon_width=32, photon_height=32, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.01)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 24, 24, sc.fov)
    other = scenes.cornell_variant(9, min_tris=500, max_tris=2000)
    bt = g.Batch(max_jobs=4)
    bt.add_job(g.default_config(16, photon_width=16, photon_height=16), other.scene.to_mesh(),
               g.look_at(other.scene.camera_origin, other.scene.camera_lookat, 16, 16, 45))
    j = bt.add_job(cfg, mesh, cam)
    bt.run_passes(7)
    ck = bt.save_checkpoint(j)
    bt.run_passes(5)
    r = setup(cfg, mesh, cam)
    r.load_checkpoint(ck)
    r.run_passes(5)
    for k in KINDS:
        assert same(bt.read_state(j, k), r.read_state(k)), k
    assert same(bt.read_image(j), r.read_image())


def test_checkpoint_of_another_size_is_rejected(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 16, 16, sc.fov)
    a = setup(g.default_config(16), mesh, cam)
    ck = a.save_checkpoint()
    b = setup(g.default_config(16, photon_width=8, photon_height=8), mesh, cam)
    with pytest.raises(N.SppmError):
        b.load_checkpoint(ck)
    with pytest.raises(N.SppmError):
        a.load_checkpoint(ck[:-4])
    bad = bytearray(ck)
    bad[0:8] = b"NOTACKPT"
    with pytest.raises(N.SppmError):
        a.load_checkpoint(bytes(bad))


def test_checkpoint_of_another_scene_camera_or_seed_is_rejected(cornell_c1_mesh):
    """A checkpoint carries fingerprints of the scene, the camera and the seed: loading it into a
    job of the same sizes that renders something else fails instead of continuing with progressive
    state that belongs to another image."""
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(16, photon_width=16, photon_height=16)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 16, 16, sc.fov)
    a = setup(cfg, mesh, cam)
    a.run_passes(3)
    ck = a.save_checkpoint()
    other = scenes.cornell_variant(4, min_tris=500, max_tris=2000).scene.to_mesh()
    b = setup(cfg, other, cam)
    with pytest.raises(N.SppmError, match="another scene"):
        b.load_checkpoint(ck)
    moved = g.look_at((sc.camera_origin[0] + 0.01, sc.camera_origin[1], sc.camera_origin[2]), sc.camera_lookat,
                      16, 16, sc.fov)
    c = setup(cfg, mesh, moved)
    with pytest.raises(N.SppmError, match="another camera"):
        c.load_checkpoint(ck)
    d = setup(g.default_config(16, photon_width=16, photon_height=16, seed_mode=N.SEED_HASH, seed=7), mesh, cam)
    with pytest.raises(N.SppmError, match="seeded"):
        d.load_checkpoint(ck)
    # the same scene, camera and seed in a fresh context still load and continue
    e = setup(cfg, mesh, cam)
    e.load_checkpoint(ck)
    a.run_passes(2)
    e.run_passes(2)
    assert same(a.read_state("flux_radius"), e.read_state("flux_radius"))
