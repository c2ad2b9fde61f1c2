"""The CPU oracle (oracle/sppm_oracle.c) equals the reference's own GLSL shaders, compiled as C++
through oracle/glsl_compat.hpp and driven like m_display (oracle/ref_shaders.cpp): the complete
per-pixel and per-photon state after every frame, word for word.

Needs the reference sources (built into oracle/_ref); skipped where they are absent (the GPU machine),
where the committed fixtures of tests/golden carry the pinned outputs instead.
"""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N
from tests.golden.fixtures import camera_from

pytestmark = pytest.mark.reference

KINDS = ["hit_position", "hit_reflectance", "hit_normal", "eye_rng", "hit_triangle", "hit_t", "emission_n",
         "flux_radius", "photon_position", "photon_flux", "photon_direction", "photon_rng", "photon_hit",
         "slot_winner", "slot_count"]


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype.itemsize == 4 else a


def compare(o, r, label):
    bad = []
    for kind in KINDS:
        a, b = bits(o.read_state(kind)), bits(r.read_state(kind))
        if a.shape != b.shape or not np.array_equal(a, b):
            bad.append((kind, int((a != b).reshape(len(a), -1).any(axis=1).sum()) if a.shape == b.shape else -1))
    assert not bad, f"{label}: oracle differs from the reference shaders: {bad}"


def run(scene, cam, R, checkpoints, textured=False, lens=None):
    from oracle.binding import Oracle
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import RefShaders
    build_ref(reference_dir())
    cfg = g.default_config(R)
    r = RefShaders(scene, cam, R)
    if lens is not None:
        cfg.focal_length, cfg.aperture = lens
        r.set_lens(*lens)
    o = Oracle(cfg, scene, cam)
    done = 0
    for k in checkpoints:
        o.run_frames(k - done)
        lookups = r.run_frames(k - done)  # texture3D calls so far
        assert (lookups > 0) == textured
        done = k
        compare(o, r, f"after {k} frames")
        s, fi = r.scalars(), o.frame_info()
        assert np.float32(s[2]) == np.float32(fi.num_photons_f32)
        assert np.float32(s[3]) == np.float32(fi.initial_radius) and np.float32(s[4]) == np.float32(fi.grid_scale)
        assert np.array_equal(s[5:8], np.array(list(fi.bbox_min), np.float32))
        assert np.array_equal(s[8:11], np.array(list(fi.bbox_max), np.float32))
    disp = o.read_image(N.IMAGE_DISPLAY).astype(np.float32)
    assert np.array_equal(bits(disp), bits(r.display()))


def test_oracle_equals_reference_shaders_cornell_metal(cornell_metal):
    arrays, d = cornell_metal
    scene = g.scene_from_arrays(arrays)
    cam = camera_from(d, 16, 16)
    run(scene, cam, 16, [1, 2, 10, 11, 21])


def test_oracle_equals_reference_shaders_cornell_box(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)
    run(mesh.scene(), cam, 32, [1, 3, 12])


@pytest.mark.parametrize("light", [True, False])
def test_oracle_equals_reference_shaders_every_material_class(light):
    """Glass, plastic, glossy metal, glossy glass and glossy plastic (and, without the light, the
    environment emission and sky of GenerateIBLSample)."""
    from glslppm_gb300 import scenes
    sc = scenes.materials_box(light=light)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)  # power of two: ReduceTexture
    run(sc.to_mesh().scene(), cam, 32, [1, 2, 11, 21])


def test_oracle_equals_reference_shaders_textured(tmp_path):
    """map_Kd textures sampled on the eye path, by photon emission from a textured light and by
    photon bounces (barycentrics from the stored position), GL_LINEAR / GL_REPEAT as
    include/sppm_texture.h pins them."""
    from glslppm_gb300 import scenes
    sc = scenes.textured_box()
    mesh = g.Mesh.load_obj(str(sc.write_obj(tmp_path / "t.obj"))).build_bvh()
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)
    run(mesh.scene(), cam, 32, [1, 2, 11, 21], textured=True)


def test_oracle_equals_reference_shaders_depth_of_field(cornell_c1_mesh):
    """A thin lens with a non-zero aperture (eyeraytrace.fs:404-421)."""
    sc, mesh = cornell_c1_mesh
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)
    run(mesh.scene(), cam, 32, [1, 11, 21], lens=(1.8, 0.06))

