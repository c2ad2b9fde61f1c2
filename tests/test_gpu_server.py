"""Continuous-batching server: requests submitted while others run are admitted as slots and
memory free up, and every result equals the single-job render of the same request, word for word
(FP32 path), whatever else was on the GPU with it."""
import threading
import time

import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N, scenes

pytestmark = pytest.mark.gpu


def requests():
    out = []
    for i, seed in enumerate((3, 4, 5, 6, 7, 8)):
        j = scenes.cornell_variant(seed, min_tris=500, max_tris=4000)
        w, h = (24, 24) if i % 2 else (32, 16)
        cfg = g.default_config(w, height=h, photon_width=32, photon_height=16 + 8 * (i % 3),
                               radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.01, seed=seed)
        sc = j.scene
        cam = g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov)
        out.append((cfg, sc.to_mesh(), cam, 5 + 7 * i))
    return out


def alone(cfg, mesh, cam, passes):
    r = g.Renderer(cfg)
    r.upload_scene(mesh)
    r.set_camera(cam)
    r.run_passes(passes)
    return r.read_image()


def test_results_equal_single_renders_in_the_mix():
    reqs = requests()
    srv = g.Server(max_jobs=3, passes_per_step=2)
    tickets = []
    for k, (cfg, mesh, cam, passes) in enumerate(reqs):
        tickets.append(srv.submit(cfg, mesh, cam, passes))
        if k % 2:
            time.sleep(0.02)  # later requests arrive while earlier ones are on the GPU
    infos = [srv.wait(t, timeout=120) for t in tickets]
    assert all(i.state == N.REQUEST_DONE for i in infos)
    for t, info, (cfg, mesh, cam, passes) in zip(tickets, infos, reqs):
        assert info.passes_done == passes and info.t_done >= info.t_admit >= info.t_submit
        img = srv.fetch_image(t)
        ref = alone(cfg, mesh, cam, passes)
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), f"ticket {t}"
    st = srv.stats()
    assert st.completed == len(reqs) and st.failed == 0 and st.resident == 0 and st.queued == 0
    # three slots for six requests: some requests waited for a slot
    assert max(i.t_admit - i.t_submit for i in infos) > 0
    srv.close()


def test_memory_budget_admits_one_at_a_time_and_rejects_oversize():
    reqs = requests()
    cfg, mesh, cam, _ = reqs[0]
    b = g.Batch(max_jobs=2)
    need = b.job_bytes(cfg, mesh)
    b.close()
    srv = g.Server(max_jobs=8, memory_budget=int(need * 1.6))
    ts = [srv.submit(cfg, mesh, cam, 6) for _ in range(3)]
    infos = [srv.wait(t, timeout=120) for t in ts]
    assert all(i.state == N.REQUEST_DONE for i in infos)
    # admitted one at a time: each waited for the previous one to finish
    assert infos[1].t_admit >= infos[0].t_done and infos[2].t_admit >= infos[1].t_done
    imgs = [srv.fetch_image(t) for t in ts]
    assert all(np.array_equal(imgs[0], x) for x in imgs[1:])
    big = g.default_config(256, photon_width=512, photon_height=512)
    with pytest.raises(N.SppmError) as e:
        srv.submit(big, mesh, g.look_at((0.5, 0.5, 2), (0.5, 0.5, 0), 256, 256, 45), 1)
    assert e.value.status == N.ERR_OOM
    srv.close()


def test_submit_from_many_threads_and_poll():
    reqs = requests()[:4]
    srv = g.Server(max_jobs=4)
    tickets, lock = [], threading.Lock()

    def client(req):
        cfg, mesh, cam, passes = req
        t = srv.submit(cfg, mesh, cam, passes)
        with lock:
            tickets.append((t, req))

    th = [threading.Thread(target=client, args=(r,)) for r in reqs]
    for x in th:
        x.start()
    for x in th:
        x.join()
    for t, (cfg, mesh, cam, passes) in tickets:
        info = srv.wait(t, timeout=120)
        assert info.state == N.REQUEST_DONE and srv.poll(t).passes_done == passes
        assert np.array_equal(srv.fetch_image(t), alone(cfg, mesh, cam, passes))
    srv.close()


def test_server_launch_shapes_keep_results():
    """A server created with non-default launch shapes (sppm_server_config.tuning) renders every
    request as a single default context does; an invalid shape fails the creation."""
    reqs = requests()[:3]
    srv = g.Server(max_jobs=2, passes_per_step=3,
                   tuning=dict(unbinned_rays=1, trace_refill_steps=8, gather_block=64, store_block=64))
    tickets = [srv.submit(cfg, mesh, cam, passes) for (cfg, mesh, cam, passes) in reqs]
    for t, (cfg, mesh, cam, passes) in zip(tickets, reqs):
        assert srv.wait(t, timeout=120).state == N.REQUEST_DONE
        img = srv.fetch_image(t)
        assert np.array_equal(img.view(np.uint32), alone(cfg, mesh, cam, passes).view(np.uint32)), f"ticket {t}"
    srv.close()
    with pytest.raises(N.SppmError) as e:
        g.Server(max_jobs=2, tuning=dict(gather_block=40))
    assert e.value.status == N.ERR_ARG


def test_a_scene_that_fails_preparation_fails_its_request_only():
    """The server's preparation workers check each scene: a request whose BVH arrays are
    inconsistent fails with SPPM_ERR_ARG, and the requests queued behind it are admitted and
    finish as usual."""
    (cfg, mesh, cam, passes), (cfg2, mesh2, cam2, passes2) = requests()[:2]
    bad = N.Scene.from_buffer_copy(mesh.scene())
    bad.num_nodes = bad.num_nodes - 2  # no longer 2 * triangles - 1
    srv = g.Server(max_jobs=2)
    t_bad = srv.submit(cfg, bad, cam, passes)
    t_ok = srv.submit(cfg2, mesh2, cam2, passes2)
    i_bad, i_ok = srv.wait(t_bad, timeout=60), srv.wait(t_ok, timeout=120)
    assert i_bad.state == N.REQUEST_FAILED and i_bad.status == N.ERR_ARG
    assert i_ok.state == N.REQUEST_DONE and i_ok.passes_done == passes2
    ref = alone(cfg2, mesh2, cam2, passes2)
    assert np.array_equal(srv.fetch_image(t_ok).view(np.uint32), ref.view(np.uint32))
    st = srv.stats()
    assert st.failed == 1 and st.completed == 1
    srv.close()
