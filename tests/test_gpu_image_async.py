"""Images read back without waiting (sppm_read_image_async / sppm_image_wait / sppm_image_query):
every image equals the one sppm_read_image returns after the same passes, with the copies of
several steps in flight beside the passes queued after them."""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import native as N

pytestmark = pytest.mark.gpu


def _renderer(sc, mesh, w, h, precision=N.PRECISION_FP32):
    cfg = g.default_config(w, height=h, photon_width=64, photon_height=64, radius_rule=N.RADIUS_DIAGONAL,
                           radius_fraction=0.01, precision=precision)
    r = g.Renderer(cfg)
    r.upload_scene(mesh.scene())
    r.set_camera(g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov))
    return r


@pytest.mark.parametrize("pinned,precision", [(True, N.PRECISION_FP32), (False, N.PRECISION_FP32),
                                              (True, N.PRECISION_MIXED)])
def test_streamed_images_equal_synchronous_reads(cornell_c1_mesh, pinned, precision):
    """Images read without waiting, radiance and display alternately, with several copies in
    flight: each equals the synchronous read of a second context after the same passes."""
    sc, mesh = cornell_c1_mesh
    a, b = _renderer(sc, mesh, 48, 40, precision), _renderer(sc, mesh, 48, 40, precision)
    steps, depth = 12, 3
    make = (lambda: g.pinned_empty((40, 48, 3), np.float32)) if pinned else (lambda: np.empty((40, 48, 3), np.float32))
    bufs = [make() for _ in range(steps)]
    tickets = []
    expect = []
    for i in range(steps):
        a.run_passes(1)
        kind = N.IMAGE_RADIANCE if i % 2 == 0 else N.IMAGE_DISPLAY
        tickets.append(a.read_image_async(bufs[i], kind))
        if i >= depth:
            a.image_wait(tickets[i - depth])
        b.run_passes(1)
        expect.append(b.read_image(kind).copy())
    a.image_wait(tickets[-1])
    assert a.image_done(tickets[-1]) and a.image_done(tickets[0])
    for i in range(steps):
        assert np.array_equal(bufs[i].view(np.uint32), expect[i].view(np.uint32)), f"step {i}"
    # a synchronous read after asynchronous ones sees the same state
    assert np.array_equal(a.read_image().view(np.uint32), b.read_image().view(np.uint32))


def test_unknown_ticket_and_bad_buffer_are_rejected(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    r = _renderer(sc, mesh, 16, 16)
    r.run_passes(1)
    with pytest.raises(N.SppmError) as e:
        r.image_wait(1)
    assert e.value.status == N.ERR_ARG
    with pytest.raises(N.SppmError):
        r.read_image_async(np.empty((16, 15, 3), np.float32))
    t = r.read_image_async(g.pinned_empty((16, 16, 3), np.float32))
    r.synchronize()
    assert r.image_done(t)


def test_more_copies_than_tickets_in_flight(cornell_c1_mesh):
    """Beyond 16 copies in flight a call waits for the oldest; every image still arrives."""
    sc, mesh = cornell_c1_mesh
    r = _renderer(sc, mesh, 32, 32)
    r.run_passes(2)
    ref = r.read_image().copy()
    bufs = [g.pinned_empty((32, 32, 3), np.float32) for _ in range(40)]
    ts = [r.read_image_async(buf) for buf in bufs]
    r.image_wait(ts[-1])
    for buf in bufs:
        assert np.array_equal(buf.view(np.uint32), ref.view(np.uint32))


def test_batch_streamed_images(cornell_c1_mesh):
    sc, mesh = cornell_c1_mesh
    b = g.Batch()
    cams = [g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov) for w, h in ((32, 32), (40, 24))]
    ids = [b.add_job(g.default_config(w, height=h, photon_width=32, photon_height=32), mesh.scene(), c)
           for (w, h), c in zip(((32, 32), (40, 24)), cams)]
    b.run_passes(3)
    bufs = [g.pinned_empty((h, w, 3), np.float32) for w, h in ((32, 32), (40, 24))]
    ts = [b.read_image_async(j, buf) for j, buf in zip(ids, bufs)]
    b.run_passes(2)  # queued behind the resolves; the copies run beside these passes
    b.image_wait(ts[1])
    assert b.image_done(ts[0])
    b.synchronize()
    # the images are those of pass 3; re-render the same jobs for 3 passes to compare
    c = g.Batch()
    ids2 = [c.add_job(g.default_config(w, height=h, photon_width=32, photon_height=32), mesh.scene(), cm)
            for (w, h), cm in zip(((32, 32), (40, 24)), cams)]
    c.run_passes(3)
    for j, buf in zip(ids2, bufs):
        assert np.array_equal(buf.view(np.uint32), c.read_image(j).view(np.uint32))


def test_streamed_images_of_a_large_image_with_few_photons(cornell_c1_mesh):
    """A 2048x2048 image with 16x16 photon slots: the resolve of each streamed image (on the copy
    stream, beside the next pass) takes longer than the next pass's photon kernels, so the next
    pass's gather must wait for it -- every streamed display and radiance image still equals the
    synchronous read after the same passes."""
    sc, mesh = cornell_c1_mesh
    w = h = 2048

    def renderer():
        cfg = g.default_config(w, height=h, photon_width=16, photon_height=16, radius_rule=N.RADIUS_DIAGONAL,
                               radius_fraction=0.01)
        r = g.Renderer(cfg)
        r.upload_scene(mesh.scene())
        r.set_camera(g.look_at(sc.camera_origin, sc.camera_lookat, w, h, sc.fov))
        return r

    a, b = renderer(), renderer()
    steps = 6
    bufs = [g.pinned_empty((h, w, 3), np.float32) for _ in range(steps)]
    tickets, expect = [], []
    for i in range(steps):
        a.run_passes(1)
        kind = N.IMAGE_DISPLAY if i % 2 == 0 else N.IMAGE_RADIANCE
        tickets.append(a.read_image_async(bufs[i], kind))
        b.run_passes(1)
        expect.append(b.read_image(kind).copy())
    for t in tickets:
        a.image_wait(t)
    for i in range(steps):
        assert np.array_equal(bufs[i].view(np.uint32), expect[i].view(np.uint32)), f"step {i}"
