"""Counting-sort photon grid (SPPM_FLAG_PHOTON_GRID, mixed precision): the sorted records against
a restatement of their encoding from the GPU's own photon records, the gathered photon counts and
flux sums against the single-precision oracle's grid estimator, the image against the
double-precision oracle's, and the batch against single contexts, word for word."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N, scenes

pytestmark = pytest.mark.gpu

F32 = np.float32


def grid_config(res, pw, passes_unused=None, **kw):
    kw.setdefault("radius_rule", N.RADIUS_DIAGONAL)
    kw.setdefault("radius_fraction", 0.005)
    flags = kw.pop("flags", 0) | N.FLAG_PHOTON_GRID
    return g.default_config(res, photon_width=pw, photon_height=pw, precision=N.PRECISION_MIXED, flags=flags, **kw)


def render(cfg, mesh, cam, passes):
    r = g.Renderer(cfg)
    r.upload_scene(mesh)
    r.set_camera(cam)
    r.run_passes(passes)
    r.synchronize()
    return r


def frac_bits(bbmin, bbmax, G):
    e = (bbmax.astype(F32) - bbmin.astype(F32)) * F32(G)
    cells = int(max(np.ceil(x) if x > 0 else 0 for x in e))
    return max(21 - int(cells + 1).bit_length(), 0)


def expected_records(pos, flux, dirn, fi, light_area):
    """The 16-byte records photon_grid.cuh writes, restated in single-precision numpy arithmetic
    (IEEE round-to-nearest, no fused operations)."""
    bbmin, bbmax = np.array(fi.bbox_min, F32), np.array(fi.bbox_max, F32)
    G = F32(fi.grid_scale)
    F = frac_bits(bbmin, bbmax, G)
    sF = F32(2.0 ** F)
    v = ((pos.astype(F32) - bbmin) * G) * sF
    ok = (v >= 0) & (v < F32(2097151.0))
    q = np.where(ok, np.floor(np.where(ok, v, 0)), 2097151).astype(np.uint64)
    lo = q[:, 0] | (q[:, 1] << np.uint64(21)) | (q[:, 2] << np.uint64(42))
    fu = F32(light_area) * F32(3.141592) if light_area != 0 else F32(1.0)
    fs = F32(1.0) / fu
    h = np.minimum(flux.astype(F32) * fs, F32(65504.0)).astype(np.float16).view(np.uint16).astype(np.uint32)
    d = dirn.astype(F32)
    s = (np.abs(d[:, 0]) + np.abs(d[:, 1])) + np.abs(d[:, 2])
    ox, oy = d[:, 0] / s, d[:, 1] / s
    neg = d[:, 2] < 0
    tx = (F32(1.0) - np.abs(oy)) * np.copysign(F32(1.0), ox)
    ty = (F32(1.0) - np.abs(ox)) * np.copysign(F32(1.0), oy)
    ox, oy = np.where(neg, tx, ox).astype(F32), np.where(neg, ty, oy).astype(F32)
    a = np.rint(ox * F32(127.0)).astype(np.int32) & 0xFF
    b = np.rint(oy * F32(127.0)).astype(np.int32) & 0xFF
    code = (a | (b << 8)).astype(np.uint32)
    rec = np.empty((len(pos), 4), np.uint32)
    rec[:, 0] = (lo & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    rec[:, 1] = (lo >> np.uint64(32)).astype(np.uint32)
    rec[:, 2] = h[:, 0] | (h[:, 1] << 16)
    rec[:, 3] = h[:, 2] | (code << 16)
    return rec, q, F


def cell_slots(q, F, split, hn):
    """The hash slot of each photon's grid cell: the reference cell split `split` times along each
    axis (q >> (F - log2 split)), Teschner's hash reduced to [0, hn) by a multiply-high."""
    Fc = F - min(int(split).bit_length() - 1, F)
    c = q >> np.uint64(Fc)
    m = np.uint64(0xFFFFFFFF)
    h = (((c[:, 0] * np.uint64(73856093)) & m) ^ ((c[:, 1] * np.uint64(19349663)) & m) ^
         ((c[:, 2] * np.uint64(83492791)) & m))
    return ((h * np.uint64(hn)) >> np.uint64(32)).astype(np.int64)


@pytest.mark.parametrize("split", [2, 1, 8])
def test_grid_records_are_the_photon_records_sorted_by_slot(cornell_c1_mesh, split):
    """Three passes of a 64x64 image with 2^14 photon slots, grid cells of 1/2 (the default), 1 and
    1/8 of the reference's: every stored photon (flux >= 0) inside the grid has exactly one
    record, in the range of the hash slot of its cell, with the encoding restated from its
    position, flux and direction; the offsets are the exclusive prefix sums of the slots' counts."""
    sc, mesh = cornell_c1_mesh
    res, pw = 64, 128
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)
    r = g.Renderer(grid_config(res, pw))
    r.upload_scene(mesh)
    r.set_camera(cam)
    r.set_tuning(grid_cell_split=split)
    for frame in range(3):
        r.run_passes(1)
        r.synchronize()
        ofs, rec = r.debug_photon_grid()
        fi = r.frame_info()
        pos = r.read_state("photon_position")[:, :3]
        flux = r.read_state("photon_flux")[:, :3]
        dirn = r.read_state("photon_direction")[:, :3]
        stored = np.nonzero(flux[:, 0] >= 0)[0]
        want, q, F = expected_records(pos[stored], flux[stored], dirn[stored], fi, mesh.scene().light_area)
        inside = np.all(q < 2097151, axis=1)
        want, q = want[inside], q[inside]
        assert len(rec) == len(want) > 1000 and inside.mean() > 0.5
        assert ofs[0] == 0 and np.all(np.diff(ofs.astype(np.int64)) >= 0) and ofs[-1] == len(rec)
        hn = pw * pw
        slots = cell_slots(q, F, split, hn)
        assert np.array_equal(np.bincount(slots, minlength=hn), np.diff(ofs.astype(np.int64)))
        order = np.lexsort((want[:, 3], want[:, 2], want[:, 1], want[:, 0], slots))
        got_slot = np.repeat(np.arange(hn), np.diff(ofs.astype(np.int64)))
        got_order = np.lexsort((rec[:, 3], rec[:, 2], rec[:, 1], rec[:, 0], got_slot))
        assert np.array_equal(want[order], rec[got_order]), f"frame {frame}: records differ"


def test_grid_gathers_the_oracles_photon_counts(cornell_c1_mesh):
    """The 256x256 workload's first pass (2^16 photons, every pixel at the initial radius): the
    number of photons each pixel gathers, recovered from N = 0.7 M, equals the single-precision
    oracle's grid estimator's for every pixel, and tau agrees to 2e-6 relative (the oracle keeps
    the reference's FP32 statistics, the GPU double-float ones).  Over 21 passes the images stay
    within 1e-4 relative RMSE."""
    from oracle.binding import Oracle
    sc, mesh = cornell_c1_mesh
    res = 256
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)
    cfg = grid_config(res, 256)
    r = render(cfg, mesh, cam, 1)
    o = Oracle(cfg, mesh.scene(), cam)
    o.run_frames(1)
    valid = r.read_state("hit_triangle") >= 0
    m_gpu = np.rint(r.read_state("stats_n") / np.float64(F32(0.7)))
    m_ora = np.rint(o.read_state("emission_n")[:, 3].astype(np.float64) / np.float64(F32(0.7)))
    assert valid.mean() > 0.5 and (m_ora[valid] > 0).mean() > 0.3
    bad = np.nonzero(m_gpu != m_ora)[0]
    assert bad.size == 0, f"{bad.size} pixels gather another photon count; first {bad[:5]}: {m_gpu[bad[:5]]} vs {m_ora[bad[:5]]}"
    tau_gpu = r.read_state("stats_tau").reshape(-1, 3)
    tau_ora = o.read_state("flux_radius")[:, :3].astype(np.float64)
    rel = np.abs(tau_gpu - tau_ora) / np.maximum(np.abs(tau_ora), 1e-30)
    assert rel[valid].max() < 2e-6, rel[valid].max()
    r.run_passes(20)
    o.run_frames(20)
    img, ref = r.read_image().astype(np.float64), o.read_image(0).reshape(res, res, 3)
    e = float(np.sqrt(np.mean((img - ref) ** 2)) / np.sqrt(np.mean(ref ** 2)))
    print(f"21 passes: relative RMSE GPU grid vs FP32 oracle grid {e:.2e}")
    assert e < 1e-4, e
    o.close()


def test_grid_image_within_one_percent_of_fp64_oracle(cornell_c1_mesh):
    """The 256x256 workload in full (2^16 photons, 64 passes) with the grid: within 1% relative
    RMSE of the double-precision oracle's grid estimator run with the same seed and random
    sequence (unquantised positions, flux and directions, FP64 sums and statistics)."""
    from oracle.binding import Oracle
    sc, mesh = cornell_c1_mesh
    res, passes = 256, 64
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)
    cfg = grid_config(res, 256)
    img = render(cfg, mesh, cam, passes).read_image().astype(np.float64)
    o = Oracle(cfg, mesh.scene(), cam, fp64=True)
    o.run_frames(passes)
    ref = o.read_image(0).reshape(res, res, 3)
    o.close()
    e = float(np.sqrt(np.mean((img - ref) ** 2)) / np.sqrt(np.mean(ref ** 2)))
    print(f"64 passes: relative RMSE GPU grid vs FP64 oracle grid {e:.2e}")
    assert np.isfinite(img).all() and e <= 0.01, e


def test_grid_batch_equals_single_contexts():
    """Three jobs of different scenes and sizes in one batch, with the grid: every job's
    statistics and image equal its single context's word for word (the flux sums are integers,
    so the order of the records within a slot cannot change them), and the same context run
    twice gives the same state."""
    specs = []
    for seed, (w, h, pw, ph) in zip((1, 2), ((24, 16, 32, 16), (32, 32, 16, 16))):
        specs.append((scenes.cornell_variant(seed, min_tris=800, max_tris=3000).scene, w, h, pw, ph))
    specs.append((scenes.cornell_box(), 40, 24, 48, 20))

    def cfg_for(w, h, pw, ph):
        return g.default_config(w, height=h, photon_width=pw, photon_height=ph, radius_rule=N.RADIUS_DIAGONAL,
                                radius_fraction=0.01, precision=N.PRECISION_MIXED, flags=N.FLAG_PHOTON_GRID)

    kinds = ["stats_n", "stats_r2", "stats_tau", "photon_position", "photon_flux"]
    b = g.Batch(precision=N.PRECISION_MIXED, max_jobs=8)
    meshes = [s[0].to_mesh() for s in specs]
    ids = [b.add_job(cfg_for(w, h, pw, ph), m, g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov))
           for (sc, w, h, pw, ph), m in zip(specs, meshes)]
    passes = 23
    b.run_passes(passes)
    b.synchronize()
    for jid, (sc, w, h, pw, ph), m in zip(ids, specs, meshes):
        cam = g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)
        runs = [render(cfg_for(w, h, pw, ph), m, cam, passes) for _ in range(2)]
        for k in kinds:
            a = np.ascontiguousarray(b.read_state(jid, k))
            for r in runs:
                assert np.array_equal(a.view(np.uint8), np.ascontiguousarray(r.read_state(k)).view(np.uint8)), \
                    f"job {jid} {k}"
        assert np.array_equal(b.read_image(jid).view(np.uint8), runs[0].read_image().view(np.uint8))
    b.close()


def test_grid_with_photon_waves_and_shapes_is_unchanged(cornell_c1_mesh):
    """The grid built from a photon pass run in waves (the store's ranks accumulate over the
    waves), under other launch shapes and with cells 1, 4 and 8 times finer than the reference's
    along each axis (the default is 2): the statistics equal the default context's word for word."""
    sc, mesh = cornell_c1_mesh
    res = 64
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)
    cfg = grid_config(res, 128)
    base = render(cfg, mesh, cam, 12)
    want = {k: base.read_state(k) for k in ("stats_n", "stats_r2", "stats_tau")}
    for tune in ({"photon_wave": 4096}, {"photon_wave": 1024, "gather_block": 64, "store_block": 64},
                 {"unbinned_rays": 1, "trace_refill_steps": 4}, {"grid_cell_split": 1}, {"grid_cell_split": 4},
                 {"grid_cell_split": 8, "photon_wave": 2048}):
        r = g.Renderer(cfg)
        r.upload_scene(mesh)
        r.set_camera(cam)
        r.set_tuning(**tune)
        r.run_passes(12)
        r.synchronize()
        for k, v in want.items():
            assert np.array_equal(r.read_state(k).view(np.uint8), v.view(np.uint8)), (tune, k)


def test_grid_and_slot_jobs_in_one_batch_equal_single_contexts():
    """A batch of mixed-precision jobs with and without the grid (one launch per stage: the
    gather runs over 8x4 pixel tiles for every job, the slot records are filled for the jobs
    without the grid only): every job's state and image equal its single context's word for
    word."""
    specs = [(scenes.cornell_variant(4, min_tris=800, max_tris=3000).scene, 32, 24, 32, 16, N.FLAG_PHOTON_GRID),
             (scenes.cornell_box(), 40, 24, 48, 20, 0),
             (scenes.cornell_variant(5, min_tris=800, max_tris=3000).scene, 24, 40, 16, 16, N.FLAG_PHOTON_GRID)]

    def cfg_for(w, h, pw, ph, flags):
        return g.default_config(w, height=h, photon_width=pw, photon_height=ph, radius_rule=N.RADIUS_DIAGONAL,
                                radius_fraction=0.01, precision=N.PRECISION_MIXED, flags=N.FLAG_GL_DEPTH_CLIP | flags)

    b = g.Batch(precision=N.PRECISION_MIXED, max_jobs=8)
    meshes = [s[0].to_mesh() for s in specs]
    cams = [g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov) for (sc, w, h, _, _, _) in specs]
    ids = [b.add_job(cfg_for(w, h, pw, ph, f), m, cam) for (sc, w, h, pw, ph, f), m, cam in zip(specs, meshes, cams)]
    passes = 21
    b.run_passes(passes)
    b.synchronize()
    for jid, (sc, w, h, pw, ph, f), m, cam in zip(ids, specs, meshes, cams):
        r = render(cfg_for(w, h, pw, ph, f), m, cam, passes)
        for k in ("stats_n", "stats_r2", "stats_tau", "hit_position"):
            assert np.array_equal(np.ascontiguousarray(b.read_state(jid, k)).view(np.uint8),
                                  np.ascontiguousarray(r.read_state(k)).view(np.uint8)), f"job {jid} {k}"
        assert np.array_equal(b.read_image(jid).view(np.uint8), r.read_image().view(np.uint8)), f"job {jid} image"
    b.close()


def test_grid_with_fp64_statistics_holds_like_double_float(cornell_c1_mesh):
    """The grid with IEEE double statistics (SPPM_FLAG_FP64_STATISTICS, the FP64 gather variant)
    and with double-float pairs gather the same photons; over 200 passes at 64x64 their images
    agree to 1e-5 relative RMSE."""
    sc, mesh = cornell_c1_mesh
    res = 64
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov)
    a = render(grid_config(res, 64), mesh, cam, 200).read_image().astype(np.float64)
    b = render(grid_config(res, 64, flags=N.FLAG_FP64_STATISTICS), mesh, cam, 200).read_image().astype(np.float64)
    e = float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))
    print(f"200 passes: grid with double-float vs FP64 statistics {e:.2e}")
    assert np.isfinite(a).all() and e < 1e-5, e
