"""ctypes binding of the CPU oracle (test infrastructure; only tests, smoke() and the CPU baseline
of bench.py use it).

``Oracle(config, scene, camera, fp64=False)`` mirrors the native Renderer's state-reading API, so a
parity test reads the same state kinds from both and compares them.  config, scene and camera are
the sppm.h structs, either the product's (glslppm_gb300.native) or the oracle's own mirror
(oracle.structs, same layout); this module never loads the product library.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import build_oracle

_LIBS: dict[str, C.CDLL] = {}

STATE = {
    "hit_position": 0, "hit_reflectance": 1, "hit_normal": 2, "eye_rng": 3, "hit_triangle": 4,
    "emission_n": 5, "flux_radius": 6, "photon_position": 7, "photon_flux": 8, "photon_direction": 9,
    "photon_rng": 10, "photon_hit": 11, "slot_winner": 12, "slot_count": 13, "hit_t": 14,
}


def load(fp64: bool = False) -> C.CDLL:
    tag = "f64" if fp64 else "f32"
    if tag not in _LIBS:
        libs = build_oracle()
        lib = C.CDLL(str(libs[tag]))
        pre = "oracle64_" if fp64 else "oracle32_"
        P = C.c_void_p
        sig = {
            "create": (P, [P, P, P]), "reset": (None, [P]), "run_frames": (C.c_int, [P, C.c_uint32]),
            "read_state": (C.c_int, [P, C.c_uint32, P, C.c_size_t]),
            "read_image": (C.c_int, [P, C.c_uint32, P, C.c_size_t]), "frame_info": (None, [P, P]),
            "hash_build": (None, [P, P, C.c_uint32, C.c_uint32, C.c_uint32, P, C.c_float, C.c_uint32, P, P]),
            "gpurnd_sequence": (None, [P, C.c_uint32, P, P]),
            "hash_of_cell": (C.c_uint32, [C.c_float, C.c_float, C.c_float, C.c_float, C.c_uint32]),
            "fpmath": (None, [C.c_int, P, P, P, C.c_size_t]),
            "trace": (None, [P, P, P, C.c_size_t, C.c_int, C.c_int, P, P]),
            "destroy": (None, [P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, pre + name)
            fn.restype = res
            fn.argtypes = args
            setattr(lib, name, fn)
        _LIBS[tag] = lib
    return _LIBS[tag]


class Oracle:
    def __init__(self, config, scene, camera, fp64: bool = False):
        self.lib = load(fp64)
        self.config = config
        self._scene = scene  # keep the arrays alive
        self._h = self.lib.create(C.addressof(config), C.addressof(scene), C.addressof(camera))
        if not self._h:
            raise RuntimeError("oracle_create rejected the configuration or scene")
        self.width, self.height = config.width, config.height
        self.P = config.photon_width * config.photon_height
        self.hash_num = config.hash_slots or self.P

    def run_frames(self, n: int) -> None:
        err = self.lib.run_frames(self._h, n)
        if err:
            raise RuntimeError(f"oracle reported error {err}")

    def reset(self) -> None:
        self.lib.reset(self._h)

    def read_state(self, kind: str) -> np.ndarray:
        npix = self.width * self.height
        k = STATE[kind]
        if kind in ("hit_triangle",):
            out = np.empty(npix, dtype=np.int32)
        elif kind == "hit_t":
            out = np.empty(npix, dtype=np.float32)
        elif kind in ("slot_winner", "slot_count"):
            out = np.empty(self.hash_num, dtype=np.uint32)
        elif kind == "photon_hit":
            out = np.empty((self.P, 2), dtype=np.int32)
        elif kind.startswith("photon_"):
            out = np.empty((self.P, 4), dtype=np.float32)
        else:
            out = np.empty((npix, 4), dtype=np.float32)
        st = self.lib.read_state(self._h, k, out.ctypes.data, out.nbytes)
        if st:
            raise RuntimeError(f"oracle read_state({kind}) failed")
        return out

    def read_image(self, kind: int = 0) -> np.ndarray:
        out = np.empty((self.height, self.width, 3), dtype=np.float64)
        if self.lib.read_image(self._h, kind, out.ctypes.data, out.size):
            raise RuntimeError("oracle read_image failed")
        return out

    def frame_info(self):
        from .structs import FrameInfo
        fi = FrameInfo()
        self.lib.frame_info(self._h, C.addressof(fi))
        return fi

    def trace(self, org: np.ndarray, dir: np.ndarray, photon: bool = True, cull: bool = False):
        """raytrace() on single rays: (closest triangle or -1, its t) per ray."""
        org = np.ascontiguousarray(org, dtype=np.float32).reshape(-1, 3)
        dir = np.ascontiguousarray(dir, dtype=np.float32).reshape(-1, 3)
        n = org.shape[0]
        tri = np.empty(n, dtype=np.int32)
        t = np.empty(n, dtype=np.float32)
        self.lib.trace(self._h, org.ctypes.data, dir.ctypes.data, n, int(photon), int(cull), tri.ctypes.data,
                       t.ctypes.data)
        return tri, t

    def close(self) -> None:
        if self._h:
            self.lib.destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def hash_build(pos: np.ndarray, flux: np.ndarray, pw: int, ph: int, hash_slots: int, bbox_min, grid_scale: float,
               flags: int) -> tuple[np.ndarray, np.ndarray]:
    lib = load(False)
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    flux = np.ascontiguousarray(flux, dtype=np.float32)
    w = np.empty(hash_slots, dtype=np.uint32)
    c = np.empty(hash_slots, dtype=np.uint32)
    bb = (C.c_float * 3)(*bbox_min)
    lib.hash_build(pos.ctypes.data, flux.ctypes.data, pw, ph, hash_slots, C.addressof(bb), grid_scale, flags,
                   w.ctypes.data, c.ctypes.data)
    return w, c


def gpurnd_sequence(seed, n: int) -> tuple[np.ndarray, np.ndarray]:
    lib = load(False)
    s = np.ascontiguousarray(seed, dtype=np.float32)
    out = np.empty(n, dtype=np.float32)
    fin = np.empty(4, dtype=np.float32)
    lib.gpurnd_sequence(s.ctypes.data, n, out.ctypes.data, fin.ctypes.data)
    return out, fin


def hash_of_cell(cell, grid_scale: float, hash_num: int) -> int:
    return int(load(False).hash_of_cell(float(cell[0]), float(cell[1]), float(cell[2]), grid_scale, hash_num))


def fpmath(fn: int, x: np.ndarray, y: np.ndarray | None = None) -> np.ndarray:
    """The pinned functions of sppm_fpmath.h evaluated by the host (fn as sppm_debug_fpmath)."""
    lib = load(False)
    x = np.ascontiguousarray(x, dtype=np.float32)
    yy = np.zeros_like(x) if y is None else np.ascontiguousarray(y, dtype=np.float32)
    out = np.empty_like(x)
    lib.fpmath(fn, x.ctypes.data, yy.ctypes.data, out.ctypes.data, x.size)
    return out


def reduce_texture(tex: np.ndarray, resolution: int, op: int) -> np.ndarray:
    """ReduceTexture restated by the oracle (op 0 min.fs, 1 max.fs, 2 sum.fs)."""
    lib = load(False)
    if not hasattr(lib, "reduce_texture"):
        fn = lib.oracle32_reduce_texture
        fn.restype = C.c_int
        fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
        lib.reduce_texture = fn
    t = np.ascontiguousarray(tex, dtype=np.float32)
    out = np.zeros(4, np.float32)
    if lib.reduce_texture(t.ctypes.data, resolution, op, out.ctypes.data):
        raise ValueError("bad resolution or op")
    return out
