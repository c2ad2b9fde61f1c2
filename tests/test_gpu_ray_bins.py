"""The photon traversal takes its ray bins in order of the mean walk their rays took since the
last reorder (longest first), reordered at a frame with an eye pass 8 or more frames after the
last reorder: the order is a permutation of the bins, follows the costs the traversal summed
exactly as sppm_debug_ray_bins states, counts every walk of the exact traversal, and changes no
result."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N

pytestmark = pytest.mark.gpu


def expected_rank(cost: np.ndarray) -> np.ndarray:
    """sppm_debug_ray_bins: descending quantised mean steps, bins without rays last, equal keys in
    bin order; cost is per position of the previous order, rank_prev maps bins to positions."""
    n = (cost & 0xFFFFFFFF).astype(np.int64)
    steps = (cost >> 32).astype(np.int64)
    mean = np.where(n > 0, steps // np.maximum(n, 1), 0)
    k = np.where(n > 0, 1 + np.minimum(254, np.where(mean < 128, mean, 128 + (mean - 128) // 8)), 0)
    return k


def renderer(sc, mesh, size=128, photons=256, **cfg):
    r = g.Renderer(g.default_config(size, photon_width=photons, photon_height=photons, radius_rule=N.RADIUS_DIAGONAL,
                                    radius_fraction=0.01, **cfg))
    r.upload_scene(mesh)
    r.set_camera(g.look_at(sc.camera_origin, sc.camera_lookat, size, size, sc.fov))
    return r


@pytest.mark.parametrize("precision", [N.PRECISION_FP32, N.PRECISION_MIXED])
def test_bins_reordered_by_mean_walk(cornell_c1_mesh, precision):
    sc, mesh = cornell_c1_mesh
    r = renderer(sc, mesh, precision=precision)
    r.set_tuning(unbinned_rays=0)
    r.run_passes(1)
    rank, cost = r.debug_ray_bins()
    nb = rank.size
    assert nb == 24 * 512
    # frame 0's reorder had no walks to go by: bin order
    assert np.array_equal(rank, np.arange(nb))
    r.run_passes(9)
    f10 = r.frame_info()
    r.run_passes(10)  # frames 10..19: their costs, under the order set at frame 10
    f20 = r.frame_info()
    rank_prev, cost = r.debug_ray_bins()
    assert np.array_equal(np.sort(rank_prev), np.arange(nb))
    # every walk of frames 10..19 counted once (the few rays with a zero direction component that
    # the exact path walks block-wide are not)
    rays = int((cost & 0xFFFFFFFF).sum())
    segs = f20.photon_segments - f10.photon_segments
    assert 0.99 * segs <= rays <= segs, (rays, segs)
    r.run_passes(1)  # frame 20: reorder, then trace
    rank, cost20 = r.debug_ray_bins()
    assert np.array_equal(np.sort(rank), np.arange(nb))
    per_bin = cost[rank_prev]  # the costs of each bin (index = bin)
    k = expected_rank(per_bin)
    order = np.lexsort((np.arange(nb), -k))  # descending key, then bin
    want = np.empty(nb, np.int64)
    want[order] = np.arange(nb)
    assert np.array_equal(rank, want)
    assert rays > 0 and k.max() > 1
    f21 = r.frame_info()
    assert int((cost20 & 0xFFFFFFFF).sum()) <= f21.photon_segments - f20.photon_segments  # restarted
    r.close()


def expected_order(cost_by_bin: np.ndarray) -> np.ndarray:
    k = expected_rank(cost_by_bin)
    order = np.lexsort((np.arange(k.size), -k))
    want = np.empty(k.size, np.int64)
    want[order] = np.arange(k.size)
    return want


def test_reorder_cadence_with_an_eye_pass_every_frame(cornell_c1_mesh):
    """With an eye pass every frame the bins are reordered at frames 7, 15, ... (8 frames apart)."""
    sc, mesh = cornell_c1_mesh
    r = renderer(sc, mesh, eye_pass_interval=1)
    r.set_tuning(unbinned_rays=0)
    r.run_passes(7)  # frames 0..6: no reorder yet
    rank, cost = r.debug_ray_bins()
    assert np.array_equal(rank, np.arange(rank.size))
    r.run_passes(1)  # frame 7: reorder by the walks of frames 0..6
    rank7, _ = r.debug_ray_bins()
    assert np.array_equal(rank7, expected_order(cost[rank]))
    assert not np.array_equal(rank7, np.arange(rank.size))
    r.run_passes(7)  # frames 8..14: the order stands
    rank14, cost14 = r.debug_ray_bins()
    assert np.array_equal(rank14, rank7)
    r.run_passes(1)  # frame 15
    rank15, _ = r.debug_ray_bins()
    assert np.array_equal(rank15, expected_order(cost14[rank14]))
    r.close()


def test_order_changes_no_result(cornell_c1_mesh):
    """Binned rays, reordered every eye-pass cycle, against rays traced in queue order: the same
    state and image bit for bit after three cycles."""
    sc, mesh = cornell_c1_mesh
    a = renderer(sc, mesh)
    a.set_tuning(unbinned_rays=0)
    b = renderer(sc, mesh)
    b.set_tuning(unbinned_rays=1)
    a.run_passes(31)
    b.run_passes(31)
    for kind in ("flux_radius", "photon_position", "photon_flux", "slot_winner", "slot_count"):
        assert np.array_equal(a.read_state(kind).view(np.uint8), b.read_state(kind).view(np.uint8)), kind
    assert np.array_equal(a.read_image().view(np.uint32), b.read_image().view(np.uint32))
    rank, cost = a.debug_ray_bins()
    assert not np.array_equal(rank, np.arange(rank.size))  # the order did change
    a.close()
    b.close()
