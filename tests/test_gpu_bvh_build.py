"""The GPU-built BVHs (locally-ordered clustering, the default, and the radix-tree linear BVH)
have the layout of the reference's threaded BVH (six preorder orderings, miss links to the node
after each subtree, boxes that contain their children) and find the same closest triangles as the
host-built exact-SAH tree; the clustered tree needs fewer node visits per ray than the radix tree."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N, scenes

pytestmark = pytest.mark.gpu


def check_layout(a):
    nn = a.node_bounds.shape[0]
    nt = (nn + 1) // 2
    tri = a.node_triangle
    leaves = np.flatnonzero(tri >= 0)
    assert len(leaves) == nt and np.array_equal(np.sort(tri[leaves]), np.arange(nt))
    for o in range(6):
        base, miss = a.order_base[o], a.order_miss[o]
        assert np.array_equal(np.sort(base), np.arange(nn)), f"ordering {o} is not a permutation"
        assert base[0] == 0
        # walk the threaded ordering: hit -> next, miss -> miss link; every node is reached once
        # when every box is "hit", and skipping a subtree lands on the node after it
        for q in range(nn):
            m = miss[q]
            if tri[base[q]] >= 0:
                assert m == q + 1
            else:
                assert m == -1 or q < m <= nn
    # a parent's box contains its children's (ordering 0: the children of q are q+1 and miss[q+1])
    b = a.node_bounds
    base0, miss0 = a.order_base[0], a.order_miss[0]
    assert np.array_equal(base0, np.arange(nn))
    for q in range(nn):
        if tri[q] >= 0:
            continue
        c1 = q + 1
        c2 = miss0[c1] if tri[c1] < 0 else c1 + 1
        for c in (c1, c2):
            assert np.all(b[q, :3] <= b[c, :3]) and np.all(b[q, 3:] >= b[c, 3:])


@pytest.mark.parametrize("builder", ["ploc", "lbvh"])
def test_gpu_bvh_layout_and_closest_hits(builder):
    sc = scenes.cornell_variant(11, min_tris=3000, max_tris=6000).scene
    host = sc.to_mesh()
    dev = g.Mesh.from_arrays(sc.positions, sc.material_ids, sc.material_array(), sc.normals).build_bvh(
        gpu=True, builder=builder)
    ad = dev.arrays()
    check_layout(ad)
    ah = host.arrays()
    assert ad.node_bounds.shape == ah.node_bounds.shape
    # the root box is the scene box in both trees
    assert np.array_equal(ad.node_bounds[0], ah.node_bounds[0])
    cfg = g.default_config(16, photon_width=16, photon_height=16)
    rng = np.random.default_rng(3)
    org = rng.uniform(0.02, 0.98, size=(20000, 3)).astype(np.float32)
    d = rng.normal(size=(20000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    out = []
    for mesh in (host, dev):
        r = g.Renderer(cfg)
        r.upload_scene(mesh)
        out.append(r.debug_trace(org, d, photon=True))
    (th, tt_h), (td, tt_d) = out
    # the same closest distance for every ray; the same triangle except at exact ties
    np.testing.assert_array_equal(tt_h.view(np.uint32), tt_d.view(np.uint32))
    assert (th == td).mean() > 0.999


def test_gpu_bvh_renders_like_the_host_bvh():
    sc = scenes.cornell_box()
    host = sc.to_mesh()
    dev = g.Mesh.from_arrays(sc.positions, sc.material_ids, sc.material_array(), sc.normals).build_bvh(gpu=True)
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 48, 48, sc.fov)
    imgs, hits = [], []
    for mesh in (host, dev):
        r = g.Renderer(g.default_config(48, photon_width=64, photon_height=64, radius_rule=N.RADIUS_DIAGONAL,
                                        radius_fraction=0.01))
        r.upload_scene(mesh)
        r.set_camera(cam)
        r.run_passes(12)
        imgs.append(r.read_image())
        hits.append(r.read_state("hit_triangle"))
    assert (hits[0] == hits[1]).mean() > 0.999
    rel = np.sqrt(((imgs[0] - imgs[1]) ** 2).mean()) / imgs[0].mean()
    assert rel < 0.02, rel


@pytest.mark.parametrize("builder", ["ploc", "lbvh"])
def test_gpu_bvh_single_triangle_and_mixed_path(builder):
    pos = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], dtype=np.float32)
    mats = np.zeros(1, dtype=g.renderer.MATERIAL_DTYPE)
    mats[0]["color"] = (0.5, 0.5, 0.5)
    m = g.Mesh.from_arrays(pos, np.zeros(1, np.int32), mats).build_bvh(gpu=True, builder=builder)
    a = m.arrays()
    assert a.node_bounds.shape == (1, 6) and a.node_triangle[0] == 0
    assert np.all(a.order_base == 0) and np.all(a.order_miss == 1)
    sc = scenes.cornell_variant(2, min_tris=2000, max_tris=3000).scene
    dev = g.Mesh.from_arrays(sc.positions, sc.material_ids, sc.material_array(), sc.normals).build_bvh(gpu=True)
    r = g.Renderer(g.default_config(24, photon_width=32, photon_height=32, precision=N.PRECISION_MIXED))
    r.upload_scene(dev)
    r.set_camera(g.look_at(sc.camera_origin, sc.camera_lookat, 24, 24, sc.fov))
    r.run_passes(3)
    r.synchronize()
    assert np.isfinite(r.read_image()).all()


def test_clustered_tree_needs_fewer_node_visits_than_the_radix_tree():
    """Locally-ordered clustering against the Morton radix tree on the batched workload's largest
    job (398k triangles): node visits per photon segment (the traversal counters), with the
    exact-SAH host tree beside them."""
    sc = scenes.cornell_variant(17).scene
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 64, 64, sc.fov)
    visits = {}
    for name in ("host", "ploc", "lbvh"):
        m = g.Mesh.from_arrays(sc.positions, sc.material_ids, sc.material_array(), sc.normals)
        m = m.build_bvh() if name == "host" else m.build_bvh(gpu=True, builder=name)
        r = g.Renderer(g.default_config(64, photon_width=256, photon_height=256, radius_rule=N.RADIUS_DIAGONAL,
                                        radius_fraction=0.005))
        r.upload_scene(m)
        r.set_camera(cam)
        r.run_passes(2)
        visits[name] = r.traversal_counters(passes=4)["nodes_per_segment"]
        r.close()
    print("nodes per photon segment:", visits)
    assert visits["ploc"] < visits["lbvh"]
