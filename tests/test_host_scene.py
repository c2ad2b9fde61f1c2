"""Scene ingest and BVH build equal the reference's host code word for word.

The reference's mesh.cpp, bvh.cpp and camera.cpp, compiled from its own sources into oracle/_ref,
load the same OBJ files; every array CGPURT::CreateTextures would pack (positions, normals,
material ids and materials, light table, node boxes and triangles, the six orderings' base ids
and miss links) must be identical.  Without the reference sources, the committed fixture of
cornell_metal.obj (made by tests/golden/make_golden.py from the reference's host code) stands in.
"""
import numpy as np
import pytest

import glslppm_gb300 as g
from glslppm_gb300 import scenes

FIELDS = ["positions", "normals", "texcoords", "material_ids", "light_triangles", "light_cdf", "bbox_min", "bbox_max",
          "node_bounds", "node_triangle", "order_base", "order_miss"]


def assert_scene_equal(ref: dict, mine):
    for k in FIELDS:
        a, b = np.asarray(ref[k]), getattr(mine, k)
        assert a.shape == b.shape, k
        assert np.array_equal(a.view(np.uint8), np.ascontiguousarray(b).view(np.uint8)), k
    assert np.float32(ref["light_area"]) == np.float32(mine.light_area)
    m = ref["materials"] if "materials" in ref else None
    if m is not None:
        for f in ("color", "eta", "brdf"):
            assert np.array_equal(m[f], mine.materials[f]), f


def test_bvh_matches_committed_reference_fixture(cornell_metal):
    arrays, d = cornell_metal
    # rebuild the BVH from the fixture's triangles with our builder
    mesh = g.Mesh.from_arrays(arrays.positions, arrays.material_ids, arrays.materials, arrays.normals).build_bvh()
    mine = mesh.arrays()
    for k in ("node_bounds", "node_triangle", "order_base", "order_miss", "light_cdf", "light_triangles"):
        assert np.array_equal(np.asarray(d[k]).view(np.uint8), getattr(mine, k).view(np.uint8)), k
    assert len(mine.node_triangle) == 71


def test_camera_matches_reference_fixture(cornell_metal):
    arrays, d = cornell_metal
    cam = g.look_at((0, 0, 13), (0, 0, 0), 512, 512, 45)
    for k in ("origin", "u", "v", "w"):
        assert np.array_equal(np.array(list(getattr(cam, k)), np.float32), d["cam_" + k]), k
    assert np.float32(cam.distance) == d["cam_distance"]


@pytest.mark.reference
def test_obj_loader_and_bvh_equal_reference_host_code_cornell_metal():
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import run_ref_host_dump
    build_ref(reference_dir())
    ref = run_ref_host_dump(reference_dir() / "cornell_metal.obj", 0.01)
    mine = g.Mesh.load_obj(str(reference_dir() / "cornell_metal.obj"), (0, 0, 0), 0.01).build_bvh().arrays()
    assert_scene_equal(ref, mine)


@pytest.mark.reference
def test_obj_loader_and_bvh_equal_reference_host_code_generated_cornell_box(tmp_path):
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import run_ref_host_dump
    build_ref(reference_dir())
    obj = scenes.cornell_box().write_obj(tmp_path / "cornell.obj")
    ref = run_ref_host_dump(obj, 1.0)
    mine = g.Mesh.load_obj(str(obj)).build_bvh().arrays()
    assert_scene_equal(ref, mine)
    assert len(mine.positions) == 7948


@pytest.mark.reference
def test_loader_quirks_equal_reference(tmp_path):
    """Materials without Ns are dropped, Ka/Kd/Ks carry over, Ke reads as Ka, face normals when an
    index lacks a normal, long lines are chunked at 79 characters, quads use 3 vertices."""
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import run_ref_host_dump
    build_ref(reference_dir())
    (tmp_path / "q.mtl").write_text(
        "newmtl a\nKd 0.5 0.25 0.125\nNs 10\n"
        "newmtl skipped\nKd 0.9 0.9 0.9\n"
        "newmtl glassy\nKs 0.5 0.5 0.5\nNs 100\n"
        "newmtl lamp\nKe 2 2 2\nNs 0\n"
        "newmtl gloss\nKs 1 1 1\nNs 40\n")
    lines = ["mtllib q.mtl\n"]
    rng = np.random.default_rng(3)
    pts = rng.random((40, 3)).astype(np.float32)
    lines += ["v %.9g %.9g %.9g\n" % tuple(map(float, p)) for p in pts]
    lines += ["vn 0 0 2\n", "vn 0 1 0\n"]
    mats = ["a\n", "glassy\n", "lamp\n", "gloss\n", "skipped\n"]
    for t in range(24):
        if t % 5 == 0:
            lines.append("usemtl " + mats[(t // 5) % len(mats)])
        a, b, c, d4 = rng.integers(1, 41, size=4)
        if t % 7 == 3:
            lines.append(f"f {a} {b} {c} {d4}\n")  # quad: first three vertices
        elif t % 11 == 5:
            lines.append(f"f {a}//1 {b} {c}//2\n")  # missing normal -> face normals everywhere
        else:
            lines.append(f"f {a}//1 {b}//2 {c}//1\n")
    lines.append("# " + "x" * 150 + "\n")  # a long comment split into chunks
    (tmp_path / "q.obj").write_text("".join(lines))
    ref = run_ref_host_dump(tmp_path / "q.obj", 2.0)
    mine = g.Mesh.load_obj(str(tmp_path / "q.obj"), (0, 0, 0), 2.0).build_bvh().arrays()
    assert_scene_equal(ref, mine)


@pytest.mark.reference
@pytest.mark.parametrize("light", [True, False])
def test_every_material_class_round_trips_through_the_reference_loader(tmp_path, light):
    """The MTL dialect of scenes.MaterialSpec.mtl makes the reference's classifier produce every
    BRDF class of materials_box; our loader gives the same arrays."""
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import run_ref_host_dump
    build_ref(reference_dir())
    spec = scenes.materials_box(light=light)
    obj = spec.write_obj(tmp_path / "m.obj")
    ref = run_ref_host_dump(obj, 1.0)
    mine = g.Mesh.load_obj(str(obj)).build_bvh().arrays()
    assert_scene_equal(ref, mine)
    assert [int(b) for b in mine.materials["brdf"]] == [m.brdf for m in spec.materials]
    assert (len(mine.light_cdf) > 0) == light


def _resample_like_reference(img):
    """gpurt.cpp:176-196: layer texel (x, y) = source texel (x * w / 512, y * h / 512)."""
    h, w = img.shape[:2]
    xs = np.arange(512) * w // 512
    ys = np.arange(512) * h // 512
    out = np.full((512, 512, 4), 255, np.uint8)
    out[..., :3] = img[ys][:, xs]
    return out


@pytest.mark.reference
def test_textured_scene_equals_reference_loader(tmp_path):
    """map_Kd PPM textures, vt coordinates on every face vertex (kept for textured materials
    only), the textures resampled to 512x512 as the reference's packing does."""
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import run_ref_host_dump
    build_ref(reference_dir())
    spec = scenes.textured_box()
    obj = spec.write_obj(tmp_path / "t.obj")
    ref = run_ref_host_dump(obj, 1.0)
    mine = g.Mesh.load_obj(str(obj)).build_bvh().arrays()
    assert_scene_equal(ref, mine)
    assert np.array_equal(ref["texcoords"].view(np.uint32), mine.texcoords.view(np.uint32))
    raw = ref["textures_raw"]
    layers = [k for k, t in enumerate(raw) if t is not None]
    assert layers == [k for k, m in enumerate(spec.materials) if m.texture is not None]
    assert [int(x) for x in mine.material_texture] == [layers.index(k) if k in layers else -1 for k in range(len(raw))]
    for k in layers:
        assert np.array_equal(mine.textures[layers.index(k)], _resample_like_reference(raw[k])), k


def _quirky_obj(tmp_path, name, pad_lines):
    """An OBJ with material switches, a second mtllib half way, missing normals, quads and long
    lines, padded with `pad_lines` long comment lines between its lines (the padding changes no
    data: a comment chunk starts with '#' or 'x')."""
    (tmp_path / "q.mtl").write_text("newmtl a\nKd 0.5 0.25 0.125\nNs 10\nnewmtl b\nKs 0.5 0.5 0.5\nNs 100\n")
    (tmp_path / "r.mtl").write_text("newmtl lamp\nKe 2 2 2\nNs 0\nnewmtl gloss\nKs 1 1 1\nNs 40\n")
    rng = np.random.default_rng(5)
    lines = ["mtllib q.mtl\n"]
    pts = rng.random((600, 3)).astype(np.float32)
    lines += ["v %.9g %.9g %.9g\n" % tuple(map(float, p)) for p in pts]
    lines += ["vn 0 0 2\n", "vn 0 1 0\n", "vn 1 0 0\n"]
    mats = ["a\n", "b\n", "lamp\n", "gloss\n", "none\n"]
    for t in range(3000):
        if t == 1500:
            lines.append("mtllib r.mtl\n")
        if t % 97 == 0:
            lines.append("usemtl " + mats[(t // 97) % len(mats)])
        a, b, c, d4 = rng.integers(1, 601, size=4)
        if t % 7 == 3:
            lines.append(f"f {a}//3 {b}//1 {c}//2 {d4}//1\n")
        elif t == 2222:
            lines.append(f"f {a}//1 {b} {c}//2\n")  # one missing normal: face normals everywhere
        else:
            lines.append(f"f {a}//1 {b}//2 {c}//3\n")
    pad = "# " + "x" * 300 + "\n"
    per_line = -(-pad_lines // len(lines))  # padding lines after each line (rounded up)
    out = []
    for line in lines:
        out.append(line)
        out.extend([pad] * per_line)
    (tmp_path / name).write_text("".join(out))
    return tmp_path / name


def test_obj_reader_threads_give_the_sequential_result(tmp_path):
    """A file above the size at which the reader splits its lines across threads gives the same
    arrays as the same lines read in one range (materials switch and an mtllib sits across the
    ranges' boundaries)."""
    small = _quirky_obj(tmp_path, "small.obj", 0)
    big = _quirky_obj(tmp_path, "big.obj", 16000)
    assert small.stat().st_size < (4 << 20) < big.stat().st_size
    a = g.Mesh.load_obj(str(small), (0, 0, 0), 1.5).arrays()
    b = g.Mesh.load_obj(str(big), (0, 0, 0), 1.5).arrays()
    for k in ("positions", "normals", "material_ids", "materials", "light_cdf", "light_triangles"):
        x, y = getattr(a, k), getattr(b, k)
        assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8)), k


@pytest.mark.reference
def test_threaded_obj_reader_equals_reference(tmp_path):
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import run_ref_host_dump
    build_ref(reference_dir())
    big = _quirky_obj(tmp_path, "big.obj", 16000)
    ref = run_ref_host_dump(big, 1.5)
    mine = g.Mesh.load_obj(str(big), (0, 0, 0), 1.5).build_bvh().arrays()
    assert_scene_equal(ref, mine)


@pytest.mark.reference
def test_drop_in_gpurt_header_with_reference_host_code(tmp_path):
    """include/sppm_gpurt.hpp compiled into the reference's own mesh.cpp/bvh.cpp/camera.cpp flattens
    the TMesh + TBVH into exactly the arrays the reference builds; without a GPU it reports
    SPPM_ERR_NO_DEVICE through its status instead of crashing."""
    import subprocess
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import read_dump, run_ref_host_dump
    from glslppm_gb300 import native as N
    exe = build_ref(reference_dir()).get("gpurt_shim")
    assert exe is not None
    out = tmp_path / "shim.bin"
    frames = 3 if N.device_count() else 2
    proc = subprocess.run([str(exe), "cornell_metal.obj", "0.01", str(out), str(frames)], cwd=str(reference_dir()),
                          capture_output=True, text=True)
    if N.device_count():
        assert proc.returncode == 0 and "rendered 3 frames" in proc.stdout
    else:
        assert proc.returncode == N.ERR_NO_DEVICE and "no CUDA device" in proc.stdout
    a, b = read_dump(out), run_ref_host_dump(reference_dir() / "cornell_metal.obj", 0.01)
    for k in FIELDS:
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(b[k]).view(np.uint8)), k


@pytest.mark.reference
def test_drop_in_gpurt_header_passes_textures(tmp_path):
    """The CGPURT shim hands the reference TMesh's map_Kd textures over as 512x512 layers, equal
    to the reference's resampling and to our own loader's."""
    import subprocess
    from oracle.build import build_ref, reference_dir
    from oracle.refdump import read_dump, run_ref_host_dump
    exe = build_ref(reference_dir()).get("gpurt_shim")
    obj = scenes.textured_box().write_obj(tmp_path / "t.obj")
    out = tmp_path / "shim.bin"
    subprocess.run([str(exe), obj.name, "1.0", str(out), "0"], cwd=str(tmp_path), check=True, capture_output=True)
    a, ref = read_dump(out), run_ref_host_dump(obj, 1.0)
    for k in FIELDS:
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(ref[k]).view(np.uint8)), k
    mine = g.Mesh.load_obj(str(obj)).arrays()
    for m, (layer, raw) in enumerate(zip(a["textures_raw"], ref["textures_raw"])):
        assert (layer is None) == (raw is None), m
        if raw is not None:
            assert np.array_equal(layer, _resample_like_reference(raw)[..., :3]), m
            assert np.array_equal(layer, mine.textures[mine.material_texture[m]][..., :3]), m


def test_cornell_variants_are_seeded_and_in_range():
    from glslppm_gb300 import scenes
    a, b = scenes.cornell_variant(7), scenes.cornell_variant(7)
    assert np.array_equal(a.scene.positions, b.scene.positions) and a.width == b.width
    sizes = set()
    for s in range(12):
        j = scenes.cornell_variant(s, min_tris=2_000, max_tris=20_000)
        n = j.scene.num_triangles
        assert 1_500 <= n <= 25_000, n
        assert j.width == j.height and j.width in (128, 256, 512, 1024)
        e = int(np.log2(j.photon_width * j.photon_height))
        assert 14 <= e <= 19 and j.photon_width in (j.photon_height, 2 * j.photon_height)
        assert j.scene.material_ids.max() < len(j.scene.materials)
        sizes.add(j.width)
    assert len(sizes) >= 3


def test_image_files(tmp_path):
    img = np.random.default_rng(0).random((5, 7, 3)).astype(np.float32) * 2.0
    img[0, 0] = (np.nan, -1.0, 0.5)
    g.write_image(tmp_path / "a.pfm", img, "pfm")
    raw = (tmp_path / "a.pfm").read_bytes()
    head = b"PF\n7 5\n-1.0\n"
    assert raw.startswith(head)
    data = np.frombuffer(raw[len(head):], dtype="<f4").reshape(5, 7, 3)
    assert np.array_equal(data.view(np.uint32), img.view(np.uint32))  # bottom row first, as stored
    g.write_image(tmp_path / "a.ppm", img, "ppm")
    raw = (tmp_path / "a.ppm").read_bytes()
    head = b"P6\n7 5\n255\n"
    assert raw.startswith(head)
    px = np.frombuffer(raw[len(head):], dtype=np.uint8).reshape(5, 7, 3)
    ref = np.round(np.clip(np.nan_to_num(img, nan=0.0), 0, 1) * 255).astype(np.uint8)[::-1]
    assert np.array_equal(px, ref)
    with pytest.raises(g.SppmError):
        g.write_image(tmp_path / "missing" / "x.pfm", img)


def _read_exr(raw: bytes):
    """Parses an uncompressed single-part scanline OpenEXR file by the format's published layout."""
    import struct
    assert struct.unpack_from("<II", raw, 0) == (20000630, 2)
    pos, attrs = 8, {}
    while raw[pos] != 0:
        name_end = raw.index(b"\0", pos)
        name = raw[pos:name_end].decode()
        type_end = raw.index(b"\0", name_end + 1)
        typ = raw[name_end + 1:type_end].decode()
        (size,) = struct.unpack_from("<I", raw, type_end + 1)
        attrs[name] = (typ, raw[type_end + 5:type_end + 5 + size])
        pos = type_end + 5 + size
    pos += 1
    chans, cl = [], attrs["channels"][1]
    q = 0
    while cl[q] != 0:
        e = cl.index(b"\0", q)
        ptype, plin, xs, ys = struct.unpack_from("<iB3xii", cl, e + 1)
        chans.append((cl[q:e].decode(), ptype, xs, ys))
        q = e + 17
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    assert attrs["compression"] == ("compression", b"\0") and attrs["lineOrder"] == ("lineOrder", b"\0")
    offsets = struct.unpack_from(f"<{h}Q", raw, pos)
    out = {c[0]: np.zeros((h, w), np.float32) for c in chans}
    for off in offsets:
        y, n = struct.unpack_from("<iI", raw, off)
        assert n == 4 * w * len(chans)
        data = np.frombuffer(raw, dtype="<f4", count=w * len(chans), offset=off + 8).reshape(len(chans), w)
        for k, c in enumerate(chans):
            out[c[0]][y - y0] = data[k]
    return chans, w, h, out


def test_exr_file(tmp_path):
    img = np.random.default_rng(1).random((6, 9, 3)).astype(np.float32) * 3.0
    img[2, 4] = (np.inf, -0.5, 1e-30)
    g.write_image(tmp_path / "a.exr", img, "exr")
    chans, w, h, planes = _read_exr((tmp_path / "a.exr").read_bytes())
    assert (w, h) == (9, 6)
    assert [c[0] for c in chans] == ["B", "G", "R"] and all(c[1:] == (2, 1, 1) for c in chans)
    top_first = img[::-1]
    for k, name in enumerate("RGB"):
        assert np.array_equal(planes[name].view(np.uint32), np.ascontiguousarray(top_first[..., k]).view(np.uint32))
