"""The C++ drop-in CGPURT (include/sppm_gpurt.hpp) driven like the reference's main()/m_display():
compiled against stand-ins of the reference's mesh.h / bvh.h / camera.h (tests/dropin, over this
library's own loader, exact-SAH builder and camera), it renders on the GPU and its radiance image
equals the ctypes path's bit for bit.  The same header compiled into the reference's own host
sources is tested in tests/test_host_scene.py where those sources are present."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
LIB = REPO / "glslppm_gb300" / "_lib"


def build_driver(tmp: Path) -> Path:
    exe = tmp / "gpurt_render"
    subprocess.run(["g++", "-std=c++14", "-O2", "-ffp-contract=off", "-Wall", f"-I{REPO / 'tests' / 'dropin'}",
                    f"-I{REPO / 'include'}", str(REPO / "tests" / "dropin" / "gpurt_render.cpp"), f"-L{LIB}", "-lsppm",
                    f"-Wl,-rpath,{LIB}", "-o", str(exe)], check=True, capture_output=True, text=True)
    return exe


def cornell_obj(tmp: Path) -> tuple:
    from glslppm_gb300 import scenes
    sc = scenes.cornell_box(segments=24, rings=12)
    return sc, sc.write_obj(tmp / "cornell.obj")


def run(exe, obj, sc, res, frames, out):
    args = [str(exe), str(obj), "1.0", str(res), str(frames), "0.005", *map(repr, map(float, sc.camera_origin)),
            *map(repr, map(float, sc.camera_lookat)), repr(float(sc.fov)), str(out)]
    return subprocess.run(args, capture_output=True, text=True, timeout=300)


def test_dropin_header_compiles_and_reports_no_device_cleanly(native_lib, tmp_path):
    if native_lib.device_count() > 0:
        pytest.skip("a GPU is visible (the GPU test renders)")
    exe = build_driver(tmp_path)
    sc, obj = cornell_obj(tmp_path)
    p = run(exe, obj, sc, 16, 1, tmp_path / "img.bin")
    assert p.returncode == 3 and f"status {native_lib.ERR_NO_DEVICE}" in p.stderr


@pytest.mark.gpu
def test_dropin_cgpurt_renders_like_the_ctypes_path(tmp_path):
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    exe = build_driver(tmp_path)
    sc, obj = cornell_obj(tmp_path)
    res, frames = 64, 12
    p = run(exe, obj, sc, res, frames, tmp_path / "img.bin")
    assert p.returncode == 0, p.stdout + p.stderr
    img = np.fromfile(tmp_path / "img.bin", dtype=np.float32).reshape(res, res, 3)
    mesh = g.Mesh.load_obj(str(obj)).build_bvh()
    r = g.Renderer(g.default_config(res, radius_rule=N.RADIUS_DIAGONAL, radius_fraction=0.005))
    r.upload_scene(mesh)
    r.set_camera(g.look_at(sc.camera_origin, sc.camera_lookat, res, res, sc.fov))
    r.run_passes(frames)
    ref = r.read_image(N.IMAGE_RADIANCE)
    assert np.isfinite(img).all() and img.max() > 0
    assert np.array_equal(img.view(np.uint32), ref.astype(np.float32).view(np.uint32))
