"""Known-answer tests of the oracle against the committed golden vectors (tests/golden), which were
made by the oracle pinned against the reference's shaders and host code (make_golden.py)."""
import numpy as np

import glslppm_gb300 as g
from oracle.binding import Oracle, gpurnd_sequence, hash_build
from tests.golden.fixtures import camera_from, load_npz


def test_xorshift_seed_tables_and_gpurnd_sequences(cornell_metal):
    arrays, d = cornell_metal
    k = load_npz("kat_rng.npz")
    o = Oracle(g.default_config(512), g.scene_from_arrays(arrays), camera_from(d, 512, 512))
    eye, pho = o.read_state("eye_rng"), o.read_state("photon_rng")
    assert np.array_equal(np.concatenate([eye[k["eye_index"]], pho[k["photon_index"]]]).view(np.uint32),
                          k["seeds"].view(np.uint32))
    for s, draws, fin in zip(k["seeds"], k["draws"], k["final_state"]):
        got, gfin = gpurnd_sequence(s, 64)
        assert np.array_equal(got.view(np.uint32), draws.view(np.uint32))
        assert np.array_equal(gfin.view(np.uint32), fin.view(np.uint32))
        assert np.all((got >= 0) & (got < 1))


def test_hashed_grid_of_a_seeded_photon_set():
    k = load_npz("kat_hash.npz")
    pw, ph = int(k["photon_width"]), int(k["photon_height"])
    for hs in (4096, 1000):
        for flags in (0, 1):
            w, c = hash_build(k["pos"], k["flux"], pw, ph, hs, k["bbox_min"], float(k["grid_scale"]), flags)
            assert np.array_equal(w, k[f"winner_{hs}_{flags}"]) and np.array_equal(c, k[f"count_{hs}_{flags}"])
            valid = k["flux"][:, 0] >= 0
            assert c.sum() == valid.sum()  # every valid photon counted once (correction.vs)


def test_depth_clip_drops_last_half_row_from_the_hash_only():
    k = load_npz("kat_hash.npz")
    pw, ph = int(k["photon_width"]), int(k["photon_height"])
    w1 = k["winner_4096_1"]
    stored = w1[w1 != 0xFFFFFFFF]
    assert not np.any(stored >= (ph - 1) * pw + pw // 2)  # scatter.vs: z >= 1 clipped
    assert np.array_equal(k["count_4096_1"], k["count_4096_0"])  # correction.vs has no clip


def test_frames_match_committed_state(cornell_metal):
    arrays, d = cornell_metal
    gold = load_npz("kat_frames_cm32.npz")
    cam = camera_from(d, 32, 32)
    cam.distance = float(gold["cam_distance_32"])
    o = Oracle(g.default_config(32), g.scene_from_arrays(arrays), cam)
    done = 0
    for kf in (1, 10, 23):
        o.run_frames(kf - done)
        done = kf
        for kind in ("hit_triangle", "hit_position", "flux_radius", "emission_n", "photon_position", "photon_flux",
                     "photon_hit", "slot_winner", "slot_count"):
            a, b = o.read_state(kind), gold[f"{kind}_{kf}"]
            assert np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8)), kind
        assert o.frame_info().photons_emitted == int(gold[f"photons_{kf}"])


def test_fp64_oracle_converges_towards_fp32(cornell_c1_mesh):
    """The double-precision restatement renders the same scene (different random stream): after
    enough passes the two images agree in the mean."""
    sc, mesh = cornell_c1_mesh
    cfg = g.default_config(32, radius_rule=1, radius_fraction=0.01)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 32, 32, sc.fov)
    o32 = Oracle(cfg, mesh.scene(), cam)
    o64 = Oracle(cfg, mesh.scene(), cam, fp64=True)
    o32.run_frames(60)
    o64.run_frames(60)
    a, b = o32.read_image(0), o64.read_image(0)
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert abs(a.mean() - b.mean()) / b.mean() < 0.1
