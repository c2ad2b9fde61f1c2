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
