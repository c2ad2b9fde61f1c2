"""Launch shapes and their autotuner (sppm_set_tuning / sppm_autotune / sppm_tune_hash_slots):
the shapes change how a pass is launched, never what it computes -- images and state under every
tuning, under tunings changed between passes and after the autotuner's own passes equal a
default context's bit for bit."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N, scenes

pytestmark = pytest.mark.gpu

KINDS = ["hit_position", "hit_triangle", "emission_n", "flux_radius", "photon_position", "photon_flux",
         "photon_hit", "slot_winner", "slot_count"]

TUNINGS = [
    dict(trace_blocks_per_sm=1),
    dict(trace_refill_steps=8),
    dict(trace_refill_steps=64, unbinned_rays=1),
    dict(gather_block=64, store_block=32, eye_block=32),
    dict(trace_blocks_per_sm=2, trace_refill_steps=5, gather_block=96, store_block=64, eye_block=96),
    dict(trace_tail_lanes=8),   # a drained warp with at most 8 walking lanes hands them over
    dict(trace_tail_lanes=32, trace_refill_steps=4),  # every drained warp hands its walks over
    dict(trace_tail_lanes=1),
    dict(wide_bvh=1),  # the plain path through the 4-wide BVH (same hits on these scenes, ties in exact order)
    dict(wide_bvh=1, trace_refill_steps=4, unbinned_rays=1, photon_wave=1024),
    dict(photon_wave=1024),  # the photon pass in three waves of at most 1024 slots
    dict(photon_wave=2048, unbinned_rays=1, trace_refill_steps=4),
]


def _renderer(sc, mesh, precision, w=48, h=40, pw=64, ph=48):
    cfg = g.default_config(w, height=h, photon_width=pw, photon_height=ph, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01, precision=precision)
    r = g.Renderer(cfg)
    r.upload_scene(mesh)
    r.set_camera(g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov))
    return r


def _state(r, precision):
    kinds = KINDS + (["stats_n", "stats_r2", "stats_tau"] if precision == N.PRECISION_MIXED else [])
    out = {k: r.read_state(k).copy() for k in kinds}
    out["image"] = r.read_image().copy()
    return out


def _same(a, b, what):
    for k in a:
        x, y = np.ascontiguousarray(a[k]), np.ascontiguousarray(b[k])
        assert x.shape == y.shape and np.array_equal(x.view(np.uint8), y.view(np.uint8)), f"{what}: {k}"


@pytest.mark.parametrize("precision", [N.PRECISION_FP32, N.PRECISION_MIXED])
def test_every_tuning_renders_the_same_bits(cornell_c1_mesh, precision):
    sc, mesh = cornell_c1_mesh
    ref = _renderer(sc, mesh, precision)
    ref.run_passes(23)
    want = _state(ref, precision)
    for t in TUNINGS:
        r = _renderer(sc, mesh, precision)
        r.set_tuning(**t)
        got = r.get_tuning()
        for k, v in t.items():
            assert getattr(got, k) == v, (t, k)
        r.run_passes(23)
        _same(want, _state(r, precision), str(t))


def test_tuning_changed_between_passes(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    ref = _renderer(sc, mesh, N.PRECISION_FP32)
    ref.run_passes(35)
    r = _renderer(sc, mesh, N.PRECISION_FP32)
    for i in range(5):
        r.set_tuning(**TUNINGS[i])
        r.run_passes(7)
    _same(_state(ref, N.PRECISION_FP32), _state(r, N.PRECISION_FP32), "tuning changed every 7 passes")


def test_defaults_reported_and_bad_shapes_rejected(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    r = _renderer(sc, mesh, N.PRECISION_FP32)
    t = r.get_tuning()
    assert t.trace_blocks_per_sm >= 1 and t.trace_refill_steps == 32
    assert (t.eye_block, t.store_block, t.gather_block, t.unbinned_rays) == (128, 128, 256, 0)
    for bad in (dict(gather_block=48), dict(eye_block=256), dict(store_block=160),
                dict(trace_blocks_per_sm=t.trace_blocks_per_sm + 1), dict(unbinned_rays=2),
                dict(trace_refill_steps=5000), dict(photon_wave=512), dict(trace_tail_lanes=33),
                dict(wide_bvh=2)):
        with pytest.raises(N.SppmError) as e:
            r.set_tuning(**bad)
        assert e.value.status == N.ERR_ARG, bad
    assert r.get_tuning().as_dict() == t.as_dict()  # a rejected tuning changes nothing


@pytest.mark.parametrize("precision", [N.PRECISION_FP32, N.PRECISION_MIXED])
def test_autotune_keeps_the_image_of_a_default_context(cornell_c1_mesh, precision):
    """The autotuner's passes are ordinary passes: the context then holds what a default context
    holds after the same number of passes."""
    sc, mesh = cornell_c1_mesh
    r = _renderer(sc, mesh, precision)
    r.run_passes(3)
    best, ms = r.autotune(1)
    assert ms > 0.0
    assert best.as_dict() == r.get_tuning().as_dict()
    r.run_passes(4)
    frames = r.frame_info().frames
    ref = _renderer(sc, mesh, precision)
    ref.run_passes(frames)
    _same(_state(ref, precision), _state(r, precision), f"autotuned {best.as_dict()}")


def test_batch_autotune_equals_single_contexts():
    specs = []
    for seed, (w, h, pw, ph) in zip((3, 4), ((32, 24, 32, 32), (24, 24, 16, 32))):
        specs.append((scenes.cornell_variant(seed, min_tris=800, max_tris=3000).scene, w, h, pw, ph))
    b = g.Batch(max_jobs=4)
    ids = []
    for sc, w, h, pw, ph in specs:
        cfg = g.default_config(w, height=h, photon_width=pw, photon_height=ph, radius_rule=N.RADIUS_DIAGONAL,
                               radius_fraction=0.01)
        ids.append(b.add_job(cfg, sc.to_mesh(), g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)))
    best, ms = b.autotune(1)
    assert ms > 0.0 and best.as_dict() == b.get_tuning().as_dict()
    b.run_passes(2)
    b.synchronize()
    for j, (sc, w, h, pw, ph) in zip(ids, specs):
        frames = b.frame_info(j).frames
        cfg = g.default_config(w, height=h, photon_width=pw, photon_height=ph, radius_rule=N.RADIUS_DIAGONAL,
                               radius_fraction=0.01)
        r = g.Renderer(cfg)
        r.upload_scene(sc.to_mesh())
        r.set_camera(g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov))
        r.run_passes(frames)
        assert np.array_equal(b.read_image(j).view(np.uint32), r.read_image().view(np.uint32)), f"job {j}"


def test_hash_slots_tuner(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(48, height=40, photon_width=64, photon_height=48, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 48, 40, sc.fov)
    slots, ms = g.tune_hash_slots(cfg, mesh, cam, passes=10)
    P = 64 * 48
    assert slots in (P, 2 * P, 4 * P)
    assert all(t > 0.0 for t in ms)
    # the chosen size runs like any configured size
    cfg.hash_slots = slots
    r = g.Renderer(cfg)
    r.upload_scene(mesh)
    r.set_camera(cam)
    r.run_passes(3)
    assert r.read_state("slot_count").size == slots


def _flat_camera(sc, w, h):
    """Every primary ray has an exact zero x component (the eye pass defers such pixels)."""
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)
    cam.u[0], cam.u[1], cam.u[2] = 0.0, 0.0, -0.5
    cam.v[0], cam.v[1], cam.v[2] = 0.0, 1.0, 0.0
    cam.w[0], cam.w[1], cam.w[2] = 0.0, 0.0, -1.0
    return cam


def _pair(cfg, scene, cam, tuning, passes=23):
    out = []
    for t in (None, tuning):
        r = g.Renderer(cfg)
        r.upload_scene(scene)
        r.set_camera(cam)
        if t:
            r.set_tuning(**t)
        r.run_passes(passes)
        out.append(_state(r, cfg.precision))
        r.close()
    _same(out[0], out[1], str(tuning))


@pytest.mark.parametrize("case", ["textured", "deferred_eye", "environment"])
def test_tuning_on_textured_deferred_and_environment_paths(tmp_path, cornell_c1_mesh, case):
    """The kernel variants with texture lookups, the eye pass's deferred-pixel list (80x64 pixels
    with zero direction components: more than the list holds) and photons from the environment,
    each under non-default shapes, against a default context."""
    tuning = dict(eye_block=32, store_block=64, gather_block=96, trace_refill_steps=5, unbinned_rays=1,
                  trace_blocks_per_sm=1)
    if case == "textured":
        sc = scenes.textured_box()
        scene = g.Mesh.load_obj(str(sc.write_obj(tmp_path / "t.obj"))).build_bvh()
        w, h = 40, 32
        cam = g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)
    elif case == "deferred_eye":
        sc, scene = cornell_c1_mesh
        w, h = 80, 64
        cam = _flat_camera(sc, w, h)
    else:
        sc = scenes.materials_box(light=False)
        scene = sc.to_mesh()
        w, h = 40, 32
        cam = g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)
    cfg = g.default_config(w, height=h, photon_width=64, photon_height=32, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01)
    _pair(cfg, scene, cam, tuning)


@pytest.mark.parametrize("precision", [N.PRECISION_FP32, N.PRECISION_MIXED])
def test_photon_waves_render_the_same_bits(cornell_c1_mesh, precision):
    """The photon pass in waves (the wavefront queue depth): 256x256 photon slots in 1, 4 and 5
    waves (the last one short), with eye passes between, give the default context's state."""
    sc, mesh = cornell_c1_mesh
    ref = _renderer(sc, mesh, precision, w=64, h=64, pw=256, ph=256)
    ref.run_passes(12)
    want = _state(ref, precision)
    for wave in (16384, 13200):
        r = _renderer(sc, mesh, precision, w=64, h=64, pw=256, ph=256)
        r.set_tuning(photon_wave=wave)
        assert r.get_tuning().photon_wave == wave
        r.run_passes(12)
        _same(want, _state(r, precision), f"photon_wave={wave}")
