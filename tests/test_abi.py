"""The C-ABI library loads and exports every function include/*.h declares (no GPU needed)."""
import re
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (REPO / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        # extern "C" declarations: <type> sppm_name(   (the static inline helpers of sppm_fpmath.h,
        # defined with SPPM_FP_FN, are header-only and not part of the exported ABI)
        for m in re.finditer(r"^(?!static|SPPM_FP_FN)[A-Za-z_][\w \t\*]*?\b(sppm_\w+)[ \t]*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("sppm_create", "sppm_upload_scene", "sppm_set_camera", "sppm_run_passes", "sppm_read_image",
                     "sppm_read_state", "sppm_last_error", "sppm_destroy", "sppm_hash_build"):
        assert required in names


def test_library_exports_every_declared_symbol(native_lib):
    lib = native_lib.lib
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert lib.sppm_abi_version() == 1


def test_python_binding_covers_every_symbol(native_lib):
    assert set(declared_functions()) <= set(native_lib.SIGNATURES), \
        set(declared_functions()) - set(native_lib.SIGNATURES)


def test_struct_layouts_match_the_header(native_lib, tmp_path):
    """ctypes mirrors of the C structs have the size and field offsets the C compiler gives them."""
    import ctypes as C
    import subprocess
    N = native_lib
    structs = {"sppm_config": N.Config, "sppm_material": N.Material, "sppm_scene": N.Scene,
               "sppm_camera": N.Camera, "sppm_frame_info": N.FrameInfo, "sppm_batch_config": N.BatchConfig,
               "sppm_batch_info": N.BatchInfo, "sppm_server_config": N.ServerConfig,
               "sppm_request_info": N.RequestInfo, "sppm_server_stats": N.ServerStats, "sppm_tuning": N.Tuning}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sppm.h"', '#include "sppm_batch.h"',
             '#include "sppm_server.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", f"-I{REPO / 'include'}", str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for cname, cls in structs.items():
        assert int(out[cname]) == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(out[f"{cname}.{fname}"]) == getattr(cls, fname).offset, f"{cname}.{fname}"


def test_config_defaults_are_the_reference_constants(native_lib):
    import glslppm_gb300 as g
    c = g.default_config(512)
    assert (c.width, c.height, c.photon_width, c.photon_height) == (512, 512, 512, 512)
    assert c.max_path_length == 10 and c.eye_pass_interval == 10
    assert c.alpha == pytest.approx(0.7) and c.initial_footprint == 2.5
    assert c.focal_length == 13.0 and c.aperture == 0.0
    assert c.flags & native_lib.FLAG_GL_DEPTH_CLIP


def test_errors_are_reported_not_raised_across_the_abi(native_lib, tmp_path):
    import glslppm_gb300 as g
    N = native_lib
    with pytest.raises(N.SppmError) as e:
        g.Mesh.load_obj(str(tmp_path / "missing.obj"))
    assert e.value.status == N.ERR_IO and "cannot open" in str(e.value)
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nf 1 2\n")
    with pytest.raises(N.SppmError) as e:
        g.Mesh.load_obj(str(bad))
    assert e.value.status == N.ERR_IO
    oob = tmp_path / "oob.obj"
    oob.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 9\n")
    with pytest.raises(N.SppmError) as e:
        g.Mesh.load_obj(str(oob))
    assert e.value.status == N.ERR_IO
    # stage entry point validates its arguments before touching the device
    import ctypes
    st = N.lib.sppm_hash_build(None, None, 4, 4, 16, (ctypes.c_float * 3)(0, 0, 0), 1.0, 0, None, None, None)
    assert st == N.ERR_ARG
    assert "null" in N.last_error()


def test_create_without_a_device_fails_cleanly(native_lib):
    import glslppm_gb300 as g
    N = native_lib
    if N.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(N.SppmError) as e:
        g.Renderer(g.default_config(16))
    assert e.value.status == N.ERR_NO_DEVICE


def test_invalid_configs_are_rejected(native_lib):
    import glslppm_gb300 as g
    N = native_lib
    for bad in (dict(width=0), dict(alpha=0.0), dict(max_path_length=0), dict(precision=9), dict(seed_mode=5),
                dict(flags=N.FLAG_PHOTON_GRID), dict(flags=N.FLAG_FP64_STATISTICS)):
        with pytest.raises(N.SppmError) as e:
            g.Renderer(g.default_config(16, **bad))
        assert e.value.status in (N.ERR_ARG, N.ERR_UNSUPPORTED)


def test_oracle_struct_mirror_matches_the_product_structs(native_lib):
    """oracle/structs.py (used where the product library must not be loaded) has the layout of the
    product's sppm.h structs, and its default configuration is sppm_config_defaults'."""
    import ctypes as C

    import glslppm_gb300 as g
    from oracle import structs as OS
    N = native_lib
    for mine, theirs in ((OS.Config, N.Config), (OS.Material, N.Material), (OS.Scene, N.Scene),
                         (OS.Camera, N.Camera), (OS.FrameInfo, N.FrameInfo)):
        assert C.sizeof(mine) == C.sizeof(theirs), mine.__name__
        assert [(f, getattr(mine, f).offset) for f, _ in mine._fields_] == \
               [(f, getattr(theirs, f).offset) for f, _ in theirs._fields_], mine.__name__
    for res in (16, 1024):
        a, b = OS.default_config(res), g.default_config(res)
        assert bytes(a) == bytes(b)


def test_cornell_box_fixture_is_the_product_scene(tmp_path):
    """The Cornell box of tests/golden/cornell_box_scene.npz (the reference's host code's loader,
    BVH and camera on the generated OBJ, made by make_golden.py) equals what the product's OBJ
    loader, BVH builder and camera make of the same OBJ, word for word -- so the CPU reference arm
    of bench.py renders exactly the GPU arm's scene without loading the product library."""
    import glslppm_gb300 as g
    from glslppm_gb300 import scenes
    from oracle.structs import camera_from_npz, scene_from_npz
    s, d = scene_from_npz(REPO / "tests" / "golden" / "cornell_box_scene.npz")
    sc = scenes.cornell_box()
    mine = g.Mesh.load_obj(str(sc.write_obj(tmp_path / "cornell_box.obj"))).build_bvh().arrays()
    for k in ("positions", "normals", "material_ids", "light_triangles", "light_cdf", "bbox_min", "bbox_max",
              "node_bounds", "node_triangle", "order_base", "order_miss"):
        a = np.ascontiguousarray(getattr(mine, k))
        b = np.ascontiguousarray(d[k])
        assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), k
    assert np.float32(mine.light_area) == np.float32(d["light_area"])
    assert np.array_equal(mine.materials["color"], d["mat_color"])
    assert np.array_equal(mine.materials["brdf"], d["mat_brdf"])
    cam = g.look_at(sc.camera_origin, sc.camera_lookat, 1024, 1024, sc.fov)
    assert bytes(cam) == bytes(camera_from_npz(d, 1024, 1024))
