"""Reader for the files written by ``ref_host_dump`` (test infrastructure).

``run_ref_host_dump`` runs the reference's own host code (compiled into ``oracle/_ref``) on an OBJ
file and returns what it built: the triangle data TMesh::LoadOBJ produced, the light table, the six
TBVH orderings and, optionally, a TCamera.  The reference opens the MTL file relative to the
current directory, so the dump runs inside the OBJ file's directory.
"""
from __future__ import annotations

import subprocess
import tempfile
from pathlib import Path

import numpy as np

from .build import REF_DIR

MATERIAL_DTYPE = np.dtype([("color", "<f4", 3), ("eta", "<f4"), ("brdf", "<i4"), ("glossiness", "<f4")])


def read_dump(path: str | Path) -> dict:
    b = Path(path).read_bytes()
    if b[:8] != b"SPPMREF1":
        raise ValueError("not a ref_host_dump file")
    off = 8

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(b, dtype=dtype, count=count, offset=off).copy()
        off += a.nbytes
        return a

    n, nm, nl, nn = (int(x) for x in take("<u4", 4))
    d = {
        "positions": take("<f4", n * 9).reshape(n, 3, 3),
        "normals": take("<f4", n * 9).reshape(n, 3, 3),
        "texcoords": take("<f4", n * 6).reshape(n, 3, 2),
        "material_ids": take("<i4", n),
        "materials": take(MATERIAL_DTYPE, nm),
        "light_triangles": take("<i4", nl),
        "light_cdf": take("<f4", nl),
        "light_area": float(take("<f4", 1)[0]),
    }
    bb = take("<f4", 6)
    d["bbox_min"], d["bbox_max"] = bb[:3].copy(), bb[3:].copy()
    d["node_bounds"] = take("<f4", nn * 6).reshape(nn, 6)
    d["node_triangle"] = take("<i4", nn)
    d["order_base"] = take("<i4", 6 * nn).reshape(6, nn)
    d["order_miss"] = take("<i4", 6 * nn).reshape(6, nn)
    cam = take("<f4", 13)
    wh = take("<u4", 2)
    d["camera"] = {"origin": cam[0:3], "u": cam[3:6], "v": cam[6:9], "w": cam[9:12], "distance": float(cam[12]),
                   "width": int(wh[0]), "height": int(wh[1])}
    # per material: textured flag, width, height and the RGB8 bytes LoadPPM read
    d["textures_raw"] = []
    for _ in range(nm):
        if off >= len(b):
            break
        textured, w, h = (int(x) for x in take("<u4", 3))
        d["textures_raw"].append(take("u1", w * h * 3).reshape(h, w, 3) if textured else None)
    return d


def run_ref_host_dump(obj: str | Path, scale: float = 1.0, camera=None) -> dict:
    """camera = (origin xyz, lookat xyz, width, height, fov) or None."""
    exe = REF_DIR / "ref_host_dump"
    if not exe.exists():
        raise FileNotFoundError(f"{exe} not built (the reference sources are needed)")
    obj = Path(obj).resolve()
    with tempfile.TemporaryDirectory() as td:
        out = Path(td) / "dump.bin"
        args = [str(exe), obj.name, repr(float(scale)), str(out)]
        if camera is not None:
            (o, l, w, h, fov) = camera
            args += [repr(float(x)) for x in o] + [repr(float(x)) for x in l] + [str(int(w)), str(int(h)), repr(float(fov))]
        subprocess.run(args, cwd=str(obj.parent), check=True, capture_output=True)
        return read_dump(out)


class RefShaders:
    """The reference's GLSL shaders compiled as C++ (oracle/_ref/libref_shaders.so), driven like
    m_display; states are returned in the layout of the oracle's read_state."""

    def __init__(self, scene, camera, resolution: int):
        import ctypes as C
        lib_path = REF_DIR / "libref_shaders.so"
        if not lib_path.exists():
            raise FileNotFoundError(f"{lib_path} not built (the reference sources are needed)")
        self.lib = C.CDLL(str(lib_path))
        P = C.c_void_p
        for name, res, args in (("ref_gl_create", P, [P, P, C.c_int]), ("ref_gl_run_frames", C.c_int, [P, C.c_uint]),
                                ("ref_gl_set_lens", None, [P, C.c_float, C.c_float]),
                                ("ref_gl_read", C.c_int, [P, C.c_int, P]), ("ref_gl_scalars", None, [P, P]),
                                ("ref_gl_display", None, [P, P]), ("ref_gl_destroy", None, [P])):
            fn = getattr(self.lib, name)
            fn.restype = res
            fn.argtypes = args
        self._scene = scene
        self.R = resolution
        self._h = self.lib.ref_gl_create(C.addressof(scene), C.addressof(camera), resolution)

    def set_lens(self, focal: float, aperture: float) -> None:
        self.lib.ref_gl_set_lens(self._h, focal, aperture)

    def run_frames(self, n: int) -> int:
        return self.lib.ref_gl_run_frames(self._h, n)  # texture3D calls (0 for untextured scenes)

    def texture(self, which: int) -> np.ndarray:
        out = np.empty((self.R * self.R, 4), np.float32)
        self.lib.ref_gl_read(self._h, which, out.ctypes.data)
        return out

    def scalars(self) -> np.ndarray:
        out = np.zeros(16, np.float32)
        self.lib.ref_gl_scalars(self._h, out.ctypes.data)
        return out

    def display(self) -> np.ndarray:
        out = np.empty((self.R, self.R, 3), np.float32)
        self.lib.ref_gl_display(self._h, out.ctypes.data)
        return out

    def _tri(self, tc: np.ndarray) -> np.ndarray:
        X = np.float32(self.scalars()[11])
        i = np.floor(tc[:, 0].astype(np.float32) * X).astype(np.int64)
        j = np.floor(tc[:, 1].astype(np.float32) * X).astype(np.int64)
        tri = (j * int(X) + i) // 6
        return np.where(tc[:, 0] < 0, -1, tri).astype(np.int32)

    def read_state(self, kind: str) -> np.ndarray:
        T = {"hit_position": 0, "hit_reflectance": 1, "hit_normal": 2, "eye_rng": 3, "emission_n": 5,
             "flux_radius": 6, "photon_position": 7, "photon_flux": 8, "photon_direction": 9, "photon_rng": 10}
        if kind in T:
            return self.texture(T[kind])
        if kind == "hit_triangle":
            return self._tri(self.texture(4))
        if kind == "hit_t":
            return self.texture(4)[:, 3].copy()
        if kind == "photon_hit":
            t = self.texture(11)
            return np.stack([self._tri(t), t[:, 2].astype(np.int32)], axis=1)
        if kind == "slot_winner":
            h = self.texture(12)
            R = np.float32(self.R)
            i = np.floor(h[:, 0] * R).astype(np.int64)
            j = np.floor(h[:, 1] * R).astype(np.int64)
            empty = (h[:, 0] == 0) & (h[:, 1] == 0)
            return np.where(empty, 0xFFFFFFFF, j * self.R + i).astype(np.uint32)
        if kind == "slot_count":
            return self.texture(13)[:, 0].astype(np.uint32)
        raise KeyError(kind)

    def close(self):
        if self._h:
            self.lib.ref_gl_destroy(self._h)
            self._h = None
