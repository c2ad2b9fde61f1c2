"""Batched SPPM: jobs advanced together by one launch per stage have, word for word, the state
that single-job contexts with the same configuration, scene and camera reach -- whatever the
other jobs in the batch, when a job joins, and after other jobs leave."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N, scenes

pytestmark = pytest.mark.gpu

KINDS = ["hit_position", "hit_triangle", "emission_n", "flux_radius", "photon_position", "photon_flux",
         "photon_rng", "photon_hit", "slot_winner", "slot_count"]


def small_jobs():
    """Three jobs of different scenes, image sizes and photon buffers (two random variants and the
    Cornell box of the main workload)."""
    out = []
    for seed, (w, h, pw, ph) in zip((1, 2), ((24, 16, 32, 16), (32, 32, 16, 16))):
        j = scenes.cornell_variant(seed, min_tris=800, max_tris=3000)
        out.append((j.scene, w, h, pw, ph))
    out.append((scenes.cornell_box(), 40, 24, 48, 20))
    return out


def config_for(w, h, pw, ph, precision=N.PRECISION_FP32, seed=0):
    return g.default_config(w, height=h, photon_width=pw, photon_height=ph, radius_rule=N.RADIUS_DIAGONAL,
                            radius_fraction=0.01, precision=precision, seed=seed)


def camera_for(sc, w, h):
    return g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)


def single_states(spec, passes, precision=N.PRECISION_FP32, kinds=KINDS):
    sc, w, h, pw, ph = spec
    r = g.Renderer(config_for(w, h, pw, ph, precision))
    r.upload_scene(sc.to_mesh())
    r.set_camera(camera_for(sc, w, h))
    r.run_passes(passes)
    r.synchronize()
    st = {k: r.read_state(k) for k in kinds}
    st["image"] = r.read_image()
    return st, r.frame_info()


def assert_same(a, b, what):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    assert a.shape == b.shape, what
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), what


@pytest.mark.parametrize("precision", [N.PRECISION_FP32, N.PRECISION_MIXED])
def test_batch_equals_single_contexts(precision):
    specs = small_jobs()
    meshes = [s[0].to_mesh() for s in specs]
    b = g.Batch(precision=precision, max_jobs=8)
    ids = [b.add_job(config_for(w, h, pw, ph, precision), m, camera_for(sc, w, h))
           for (sc, w, h, pw, ph), m in zip(specs, meshes)]
    passes = 23  # three eye passes
    b.run_passes(passes)
    b.synchronize()
    kinds = KINDS + (["stats_n", "stats_r2", "stats_tau"] if precision == N.PRECISION_MIXED else [])
    for jid, spec in zip(ids, specs):
        ref, fi_ref = single_states(spec, passes, precision, kinds)
        for k in kinds:
            assert_same(b.read_state(jid, k), ref[k], f"job {jid} {k}")
        assert_same(b.read_image(jid), ref["image"], f"job {jid} image")
        fi = b.frame_info(jid)
        assert fi.frames == fi_ref.frames == passes
        assert fi.photons_emitted == fi_ref.photons_emitted
        assert fi.photon_segments == fi_ref.photon_segments
    info = b.info()
    assert info.num_jobs == 3 and info.frames == passes
    assert info.photon_slots == sum(s[3] * s[4] for s in specs)
    # one launch per stage: the batch launched as many kernels as one single-job context
    assert info.kernel_launches == fi_ref.kernel_launches


def test_jobs_joining_and_leaving_keep_their_own_schedule():
    specs = small_jobs()
    b = g.Batch(max_jobs=4)
    (sa, wa, ha, pwa, pha), (sb, wb, hb, pwb, phb), (sc_, wc, hc, pwc, phc) = specs
    a = b.add_job(config_for(wa, ha, pwa, pha), sa.to_mesh(), camera_for(sa, wa, ha))
    c = b.add_job(config_for(wc, hc, pwc, phc), sc_.to_mesh(), camera_for(sc_, wc, hc))
    b.run_passes(7)
    j = b.add_job(config_for(wb, hb, pwb, phb), sb.to_mesh(), camera_for(sb, wb, hb))  # joins at batch frame 7
    b.run_passes(6)
    b.remove_job(c)  # leaves
    b.run_passes(9)
    b.synchronize()
    ref_a, _ = single_states(specs[0], 22)
    ref_j, _ = single_states(specs[1], 15)
    for k in KINDS:
        assert_same(b.read_state(a, k), ref_a[k], f"job a {k}")
        assert_same(b.read_state(j, k), ref_j[k], f"joined job {k}")
    assert b.frame_info(j).frames == 15 and b.frame_info(j).eye_samples == 2
    # all jobs' counters in one call equal the one-job calls, field by field
    many = b.frame_infos([j, a, a])
    for got, want in zip(many, [b.frame_info(j), b.frame_info(a), b.frame_info(a)]):
        for name, _ in N.FrameInfo._fields_:
            assert getattr(got, name) == getattr(want, name) or name in ("bbox_min", "bbox_max", "aa_offset"), name
        assert list(got.bbox_min) == list(want.bbox_min) and list(got.aa_offset) == list(want.aa_offset)
    with pytest.raises(N.SppmError):
        b.frame_infos([a, c])  # c has left
    with pytest.raises(N.SppmError):
        b.read_state(c, "hit_position")
    # the freed slot is reused
    assert b.add_job(config_for(wc, hc, pwc, phc), sc_.to_mesh(), camera_for(sc_, wc, hc)) == c


def test_admission_by_memory_budget():
    sc, w, h, pw, ph = small_jobs()[2]
    mesh = sc.to_mesh()
    cfg = config_for(w, h, pw, ph)
    probe = g.Batch(max_jobs=2)
    need = probe.job_bytes(cfg, mesh)
    probe.close()
    b = g.Batch(max_jobs=8, memory_budget=int(need * 2.5))
    b.add_job(cfg, mesh, camera_for(sc, w, h))
    b.add_job(cfg, mesh, camera_for(sc, w, h))
    with pytest.raises(N.SppmError) as e:
        b.add_job(cfg, mesh, camera_for(sc, w, h))
    assert e.value.status == N.ERR_OOM
    info = b.info()
    assert info.num_jobs == 2 and info.bytes_used <= info.memory_budget


def test_batch_rejects_mismatched_jobs():
    sc, w, h, pw, ph = small_jobs()[2]
    b = g.Batch(precision=N.PRECISION_FP32, max_jobs=2)
    with pytest.raises(N.SppmError):
        b.add_job(config_for(w, h, pw, ph, precision=N.PRECISION_MIXED), sc.to_mesh(), camera_for(sc, w, h))
    cfg = config_for(w, h, pw, ph)
    cfg.eye_pass_interval = 5
    with pytest.raises(N.SppmError):
        b.add_job(cfg, sc.to_mesh(), camera_for(sc, w, h))


def test_watchdog_error_names_the_job_whose_rays_raised_it(cornell_metal):
    """One job's BVH links form a cycle: its traversals hit their step bound and the batch reports
    that job (not another job whose rays the same warps traced next); once it is removed the
    other job runs on without an error.  (The mixed path's 4-wide tree is built from the links at
    upload, which rejects such a scene.)"""
    precision = N.PRECISION_FP32
    arrays, d = cornell_metal
    from tests.golden.fixtures import camera_from
    bad = g.renderer.SceneArrays(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                                    for k, v in arrays.__dict__.items()})
    internal = bad.node_triangle[bad.order_base] < 0
    bad.order_miss[internal] = 0  # back to the root
    cam = camera_from(d, 16, 16)
    b = g.Batch(precision=precision, max_jobs=4)
    cfg = g.default_config(16, precision=precision)
    good = b.add_job(cfg, arrays, cam)
    broken = b.add_job(cfg, bad, cam)
    b.run_passes(2)
    with pytest.raises(N.SppmError) as e:
        b.synchronize()
    assert e.value.status == N.ERR_WATCHDOG
    assert f"job {broken}:" in str(e.value), str(e.value)
    b.remove_job(broken)
    b.run_passes(2)
    b.synchronize()
    assert b.frame_info(good).frames == 4


@pytest.mark.parametrize("precision", [N.PRECISION_FP32, N.PRECISION_MIXED])
def test_textured_and_untextured_jobs_in_one_batch(tmp_path, precision):
    """A textured job makes the batch launch the kernel variants with texture lookups for every
    job: each job still has the state of its own single-job context."""
    tex = scenes.textured_box()
    tex_mesh = g.Mesh.load_obj(str(tex.write_obj(tmp_path / "t.obj"))).build_bvh()
    plain = scenes.cornell_box(16, 8)
    plain_mesh = plain.to_mesh()
    w, h = 32, 24
    cfg = config_for(w, h, 32, 32, precision)
    b = g.Batch(precision=precision, max_jobs=4)
    jt = b.add_job(cfg, tex_mesh, camera_for(tex, w, h))
    jp = b.add_job(cfg, plain_mesh, camera_for(plain, w, h))
    b.run_passes(12)
    b.synchronize()
    for j, mesh, spec in ((jt, tex_mesh, tex), (jp, plain_mesh, plain)):
        r = g.Renderer(cfg)
        r.upload_scene(mesh)
        r.set_camera(camera_for(spec, w, h))
        r.run_passes(12)
        r.synchronize()
        for k in KINDS:
            assert_same(b.read_state(j, k), r.read_state(k), f"job {j} {k}")



def test_cameras_set_in_one_call_equal_one_by_one():
    """sppm_batch_set_cameras between passes gives, bit for bit, what sppm_batch_set_camera per
    job gives; a list with an unknown or repeated id fails whole and changes no camera."""
    specs = small_jobs()
    meshes = [s[0].to_mesh() for s in specs]

    def moved(sc, w, h, step):
        o = tuple(c + 0.01 * step * (i + 1) for i, c in enumerate(sc.camera_origin))
        return g.look_at(o, sc.camera_lookat, w, h, sc.fov)

    batches = []
    for _ in range(2):
        b = g.Batch(max_jobs=8)
        ids = [b.add_job(config_for(w, h, pw, ph), m, camera_for(sc, w, h))
               for (sc, w, h, pw, ph), m in zip(specs, meshes)]
        batches.append((b, ids))
    (a, ia), (c, ic) = batches
    for step in range(1, 4):
        cams = [moved(sc, w, h, step) for (sc, w, h, pw, ph) in specs]
        a.set_cameras(ia, cams)
        for j, cam in zip(ic, cams):
            c.set_camera(j, cam)
        a.run_passes(4)
        c.run_passes(4)
    bad = [moved(sc, w, h, 9) for (sc, w, h, pw, ph) in specs]
    for ids in ([ia[0], 7, ia[2]], [ia[0], ia[1], ia[0]]):
        with pytest.raises(N.SppmError) as e:
            a.set_cameras(ids, bad)
        assert e.value.status == N.ERR_ARG
    a.run_passes(11)
    c.run_passes(11)
    for ja, jc in zip(ia, ic):
        assert_same(a.read_image(ja), c.read_image(jc), f"job {ja} image")
        assert_same(a.read_state(ja, "hit_position"), c.read_state(jc, "hit_position"), f"job {ja} hits")


def test_prepared_scene_jobs_equal_plain_jobs():
    """A scene prepared ahead of time (sppm_scene_prepare) and added to two jobs, one of them with
    random-state tables prepared ahead too (sppm_state_prepare), gives, word for word, the state of
    the same job added from the scene itself; the source arrays may be gone; tables of another
    configuration are refused."""
    sc = scenes.cornell_variant(3, min_tris=800, max_tris=3000).scene
    w, h, pw, ph = 24, 16, 32, 16
    mesh = sc.to_mesh()
    prep = g.PreparedScene(mesh)
    del mesh
    b = g.Batch(precision=N.PRECISION_MIXED, max_jobs=4)
    cfg = config_for(w, h, pw, ph, N.PRECISION_MIXED)
    cam = camera_for(sc, w, h)
    seeds = g.PreparedState(cfg)
    ids = [b.add_job_prepared(cfg, prep, cam), b.add_job_prepared(cfg, prep, cam, seeds),
           b.add_job(cfg, sc.to_mesh(), cam)]
    prep.close()
    seeds.close()
    other = N.Config.from_buffer_copy(cfg)
    other.seed = 99
    with pytest.raises(N.SppmError):
        b.add_job_prepared(cfg, g.PreparedScene(sc.to_mesh()), cam, g.PreparedState(other))
    b.run_passes(13)
    b.synchronize()
    for k in KINDS + ["stats_n", "stats_r2", "stats_tau"]:
        ref = b.read_state(ids[2], k)
        for j in ids[:2]:
            assert_same(b.read_state(j, k), ref, f"job {j} {k}")
    b.close()
