"""Parity of the CUDA FP32 path with the CPU oracle (bit-exact state after K frames).

Every per-pixel and per-photon array of the progressive state -- hit points, hit triangle ids,
(emission, N), (tau, R), photon records, the hashed grid's winner and count per slot -- is compared
word for word after several frames, including eye passes (every 10th frame) and the frame-0
initialisation.  The radiance image (re.fs) is compared exactly as well.
"""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N
from oracle.binding import Oracle, fpmath
from tests.golden.fixtures import camera_from, load_npz

pytestmark = pytest.mark.gpu

KINDS = ["hit_position", "hit_reflectance", "hit_normal", "eye_rng", "hit_triangle", "hit_t", "emission_n",
         "flux_radius", "photon_position", "photon_flux", "photon_direction", "photon_rng", "photon_hit",
         "slot_winner", "slot_count"]


def bits(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype.itemsize == 4 else a.view(np.uint8)


def assert_same(kind, gpu, cpu):
    gb, cb = bits(gpu), bits(cpu)
    assert gb.shape == cb.shape, f"{kind}: shape {gb.shape} vs {cb.shape}"
    bad = np.nonzero(gb.reshape(len(gb), -1) != cb.reshape(len(cb), -1))[0]
    assert bad.size == 0, (f"{kind}: {np.unique(bad).size} of {len(gb)} elements differ; first {bad[:5]}: "
                           f"gpu {gpu[bad[:3]]} cpu {cpu[bad[:3]]}")


def run_pair(cfg, scene, cam, checkpoints):
    r = g.Renderer(cfg)
    r.upload_scene(scene)
    r.set_camera(cam)
    o = Oracle(cfg, scene, cam)
    done = 0
    for k in checkpoints:
        r.run_passes(k - done)
        o.run_frames(k - done)
        done = k
        r.synchronize()
        for kind in KINDS:
            assert_same(f"{kind} after {k} frames", r.read_state(kind), o.read_state(kind))
        fg, fo = r.frame_info(), o.frame_info()
        assert fg.frames == fo.frames == k
        assert fg.photons_emitted == fo.photons_emitted
        assert fg.num_photons_f32 == fo.num_photons_f32
        assert fg.eye_samples == fo.eye_samples
        assert fg.grid_scale == fo.grid_scale and fg.initial_radius == fo.initial_radius
        assert list(fg.bbox_min) == list(fo.bbox_min) and list(fg.bbox_max) == list(fo.bbox_max)
        assert fg.photon_segments == fo.photon_segments and fg.eye_segments == fo.eye_segments
        img = r.read_image(N.IMAGE_RADIANCE)
        ref = o.read_image(0).astype(np.float32)
        assert_same(f"radiance after {k} frames", img.reshape(-1, 3), ref.reshape(-1, 3))
    return r, o


def test_state_bit_exact_cornell_metal(cornell_metal):
    arrays, d = cornell_metal
    scene = g.scene_from_arrays(arrays)
    cfg = g.default_config(32)
    cam = camera_from(d, 32, 32)
    cam.distance = float(load_npz("kat_frames_cm32.npz")["cam_distance_32"])
    run_pair(cfg, scene, cam, [1, 10, 11, 23])


def test_state_bit_exact_cornell_box_diagonal_radius(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(48, photon_width=64, photon_height=32, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.005)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 48, 48, sc.fov)
    run_pair(cfg, mesh.scene(), cam, [1, 12, 30])


def test_fused_photon_kernel_bit_exact(cornell_c1_mesh):
    """The single-kernel photon pass (SPPM_FLAG_FUSED_PHOTON) and the default wavefront
    (generate -> persistent trace -> store) produce the same state."""
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(32, photon_width=64, photon_height=64, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01)
    cfg.flags |= N.FLAG_FUSED_PHOTON
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)
    run_pair(cfg, mesh.scene(), cam, [1, 11])


def test_unbinned_photon_rays_bit_exact(cornell_c1_mesh):
    """Tracing the photon rays in queue order (SPPM_FLAG_UNBINNED_RAYS) instead of binned by
    direction class and origin cell changes only the order of work: the state is the same."""
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(32, photon_width=64, photon_height=64, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01)
    cfg.flags |= N.FLAG_UNBINNED_RAYS
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)
    run_pair(cfg, mesh.scene(), cam, [1, 11])


def flat_camera(sc, w, h):
    """A camera whose basis vectors have no x component: every primary eye ray lies in the plane
    x = origin.x, so each has an exact zero direction component (a degenerate slab test)."""
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)
    cam.u[0], cam.u[1], cam.u[2] = 0.0, 0.0, -0.5
    cam.v[0], cam.v[1], cam.v[2] = 0.0, 1.0, 0.0
    cam.w[0], cam.w[1], cam.w[2] = 0.0, 0.0, -1.0
    return cam


@pytest.mark.parametrize("w,h", [(32, 32), (80, 64)])
def test_eye_rays_with_zero_direction_components_bit_exact(cornell_c1_mesh, w, h):
    """Eye rays with a zero direction component are deferred to the block-wide eye pass (at most
    4096 pixels a frame; the 80x64 image has more, and the rest are walked one per thread): the
    state equals the oracle's either way."""
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(w, height=h, photon_width=64, photon_height=32, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01)
    run_pair(cfg, mesh.scene(), flat_camera(sc, w, h), [1, 10, 11, 21])


@pytest.mark.parametrize("light", [True, False])
def test_state_bit_exact_every_material_class(light):
    """Glass, plastic, glossy metal, glossy glass and glossy plastic surfaces; without the light,
    photons from the environment (GenerateIBLSample) and the sky seen by escaping eye rays."""
    from glslppm_gb300 import scenes
    sc = scenes.materials_box(light=light)
    cfg = g.default_config(40, height=32, photon_width=64, photon_height=32, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 40, 32, sc.fov)
    run_pair(cfg, sc.to_mesh().scene(), cam, [1, 10, 11, 21])


@pytest.mark.parametrize("fused", [False, True])
def test_state_bit_exact_textured(tmp_path, fused):
    """map_Kd textures read through the OBJ loader: the eye path, emission from a textured light
    and photon bounces look them up (GL_LINEAR / GL_REPEAT as include/sppm_texture.h pins it)."""
    from glslppm_gb300 import scenes
    sc = scenes.textured_box()
    mesh = g.Mesh.load_obj(str(sc.write_obj(tmp_path / "t.obj"))).build_bvh()
    cfg = g.default_config(40, height=32, photon_width=64, photon_height=32, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01)
    if fused:
        cfg.flags |= N.FLAG_FUSED_PHOTON
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 40, 32, sc.fov)
    run_pair(cfg, mesh.scene(), cam, [1, 10, 11, 21])


def test_state_bit_exact_depth_of_field(cornell_c1_mesh):
    """A thin lens with a non-zero aperture focused inside the box."""
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(40, height=32, photon_width=64, photon_height=32, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01)
    cfg.focal_length, cfg.aperture = 1.8, 0.06
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 40, 32, sc.fov)
    run_pair(cfg, mesh.scene(), cam, [1, 11, 21])


def test_state_bit_exact_non_square_and_hash_seed(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(40, height=24, photon_width=48, photon_height=20, hash_slots=1500,
                           seed_mode=N.SEED_HASH, seed=7, flags=0, eye_pass_interval=4)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 40, 24, sc.fov)
    run_pair(cfg, mesh.scene(), cam, [1, 5, 9])


def test_matches_committed_golden_frames(cornell_metal):
    """The GPU state equals the oracle outputs committed in tests/golden (generated on another
    machine): a check that neither side drifted."""
    arrays, d = cornell_metal
    gold = load_npz("kat_frames_cm32.npz")
    cfg = g.default_config(32)
    cam = camera_from(d, 32, 32)
    cam.distance = float(gold["cam_distance_32"])
    r = g.Renderer(cfg)
    r.upload_scene(arrays)
    r.set_camera(cam)
    done = 0
    for k in (1, 10, 23):
        r.run_passes(k - done)
        done = k
        for kind in ("hit_triangle", "hit_position", "flux_radius", "emission_n", "photon_position", "photon_flux",
                     "photon_hit", "slot_winner", "slot_count"):
            assert_same(f"{kind}_{k}", r.read_state(kind), gold[f"{kind}_{k}"])
        assert r.frame_info().photons_emitted == int(gold[f"photons_{k}"])


def test_fpmath_device_equals_host():
    rng = np.random.default_rng(5)
    x = np.concatenate([np.linspace(-10, 10, 20001, dtype=np.float32), rng.random(20000, dtype=np.float32) * 6.3])
    for fn in (0, 1, 3, 5):
        assert np.array_equal(bits(g.renderer.debug_fpmath(fn, x)), bits(fpmath(fn, x))), fn
    xp = rng.random(40000, dtype=np.float32)
    yp = (rng.random(40000, dtype=np.float32) * 3).astype(np.float32)
    assert np.array_equal(bits(g.renderer.debug_fpmath(2, xp, yp)), bits(fpmath(2, xp, yp)))
    assert np.array_equal(bits(g.renderer.debug_fpmath(4, xp + 1e-3)), bits(fpmath(4, xp + 1e-3)))


def test_watchdog_on_cyclic_bvh_links(cornell_metal):
    """Corrupt miss links that form a cycle: every traversal hits its step bound, the kernel
    records the error and returns, and the context stays usable (no hang, no fault)."""
    arrays, d = cornell_metal
    bad = g.renderer.SceneArrays(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                                    for k, v in arrays.__dict__.items()})
    internal = bad.node_triangle[bad.order_base] < 0  # [6, nn] positions holding internal nodes
    bad.order_miss[internal] = 0  # back to the root
    cfg = g.default_config(16)
    cam = camera_from(d, 16, 16)
    r = g.Renderer(cfg)
    r.upload_scene(bad)
    r.set_camera(cam)
    r.run_passes(2)
    with pytest.raises(N.SppmError) as e:
        r.synchronize()
    assert e.value.status == N.ERR_WATCHDOG
    # the device is still healthy: a clean scene renders on a new context
    ok = g.Renderer(cfg)
    ok.upload_scene(arrays)
    ok.set_camera(cam)
    ok.run_passes(2)
    ok.synchronize()


def test_hash_build_stage_entry_point_matches_oracle_and_golden():
    """sppm_hash_build (hash.fs + scatter.vs depth test + correction.vs blend) on caller device
    arrays: winners and counts bit-equal the oracle and the committed golden grid."""
    torch = pytest.importorskip("torch")
    from oracle.binding import hash_build as oracle_hash_build
    k = load_npz("kat_hash.npz")
    pw, ph = int(k["photon_width"]), int(k["photon_height"])
    pos = torch.from_numpy(k["pos"]).cuda()
    flux = torch.from_numpy(k["flux"]).cuda()
    stream = torch.cuda.current_stream()
    for hs in (4096, 1000):
        for flags in (0, 1):
            w = torch.empty(hs, dtype=torch.int32, device="cuda")
            c = torch.empty(hs, dtype=torch.int32, device="cuda")
            g.renderer.hash_build(pos.data_ptr(), flux.data_ptr(), pw, ph, hs, k["bbox_min"], float(k["grid_scale"]),
                                  flags, w.data_ptr(), c.data_ptr(), stream.cuda_stream)
            stream.synchronize()
            wg = w.cpu().numpy().view(np.uint32)
            cg = c.cpu().numpy().view(np.uint32)
            assert np.array_equal(wg, k[f"winner_{hs}_{flags}"]) and np.array_equal(cg, k[f"count_{hs}_{flags}"])
            wo, co = oracle_hash_build(k["pos"], k["flux"], pw, ph, hs, k["bbox_min"], float(k["grid_scale"]), flags)
            assert np.array_equal(wg, wo) and np.array_equal(cg, co)
