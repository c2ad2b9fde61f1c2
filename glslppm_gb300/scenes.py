"""Seeded synthetic scenes for the benchmark and parity workloads.

The reference renders whatever OBJ it is given (``cornell_metal.obj`` by default).  The workloads
here are generated, deterministic, and can be written as OBJ/MTL text that the reference loader
accepts (lines shorter than 80 characters, ``f a//n b//n c//n``), or handed to the native library
directly as flat arrays.

* ``cornell_box()``: the unit-cube Cornell box of the 256x256 / 1024x1024 workloads -- five
  Lambertian walls as ten triangles (red 0.63,0.06,0.05 / green 0.14,0.45,0.09 / white 0.73), a
  0.25 x 0.25 ceiling light of emission 15 as two triangles, and two 64x32-segment UV spheres
  (3,968 triangles each), one mirror and one diffuse 0.73: 7,948 triangles.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .renderer import MATERIAL_DTYPE

BRDF_LIGHT, BRDF_MATTE, BRDF_MIRROR = -1, 0, 1


@dataclass
class MaterialSpec:
    name: str
    brdf: int
    color: tuple  # final albedo / emission as the renderer uses it
    eta: float = 1.7
    glossiness: float = 0.0

    def mtl(self) -> str:
        """MTL block that the reference loader classifies into this material (mesh.cpp:520-611)."""
        if self.brdf == BRDF_LIGHT:
            ka, kd, ks, ns = (1.0, 1.0, 1.0), self.color, (0.0, 0.0, 0.0), 0.0
        elif self.brdf == BRDF_MIRROR:
            ka, kd, ks, ns = (0.0, 0.0, 0.0), self.color, (1.0, 1.0, 1.0), 100.0
        else:  # the loader scales Lambertian albedo by 0.9
            ka, kd, ks, ns = (0.0, 0.0, 0.0), tuple(c / 0.9 for c in self.color), (0.0, 0.0, 0.0), 100.0
        f = lambda v: " ".join("%.9g" % x for x in v)
        return f"newmtl {self.name}\nKa {f(ka)}\nKd {f(kd)}\nKs {f(ks)}\nNs {ns:.1f}\n"


@dataclass
class SceneSpec:
    positions: np.ndarray  # [n, 3, 3] float32
    normals: np.ndarray  # [n, 3, 3] float32
    material_ids: np.ndarray  # [n] int32
    materials: list = field(default_factory=list)
    camera_origin: tuple = (0.5, 0.5, 2.15)
    camera_lookat: tuple = (0.5, 0.5, 0.0)
    fov: float = 45.0

    @property
    def num_triangles(self) -> int:
        return int(self.positions.shape[0])

    def material_array(self) -> np.ndarray:
        a = np.zeros(len(self.materials), dtype=MATERIAL_DTYPE)
        for i, m in enumerate(self.materials):
            a[i]["color"] = m.color
            a[i]["eta"] = m.eta
            a[i]["brdf"] = m.brdf
            a[i]["glossiness"] = m.glossiness
        return a

    def to_mesh(self):
        from .renderer import Mesh
        return Mesh.from_arrays(self.positions, self.material_ids, self.material_array(), self.normals).build_bvh()

    def write_obj(self, path: str | Path) -> Path:
        """OBJ + MTL (same stem) in the dialect of the reference loader."""
        path = Path(path)
        mtl = path.with_suffix(".mtl")
        mtl.write_text("".join(m.mtl() + "\n" for m in self.materials))
        lines = [f"mtllib {mtl.name}\n"]
        n = self.num_triangles
        p = self.positions.reshape(-1, 3)
        nr = self.normals.reshape(-1, 3)
        lines += ["v %.9g %.9g %.9g\n" % tuple(map(float, v)) for v in p]
        lines += ["vn %.9g %.9g %.9g\n" % tuple(map(float, v)) for v in nr]
        cur = None
        for t in range(n):
            m = int(self.material_ids[t])
            if m != cur:
                lines.append(f"usemtl {self.materials[m].name}\n")
                cur = m
            a, b, c = 3 * t + 1, 3 * t + 2, 3 * t + 3
            lines.append(f"f {a}//{a} {b}//{b} {c}//{c}\n")
        for ln in lines:
            if len(ln) > 79:
                raise ValueError(f"OBJ line longer than the reference loader's 79-character chunks: {ln!r}")
        path.write_text("".join(lines))
        return path


def _quad(p0, p1, p2, p3, n):
    """two triangles (p0,p1,p2), (p0,p2,p3); counter-clockwise seen from the side n points to."""
    tris = np.array([[p0, p1, p2], [p0, p2, p3]], dtype=np.float64)
    e = np.cross(tris[0, 1] - tris[0, 0], tris[0, 2] - tris[0, 0])
    if np.dot(e, n) < 0:
        tris = tris[:, ::-1]
    nrm = np.broadcast_to(np.asarray(n, dtype=np.float64), (2, 3, 3))
    return tris, nrm


def uv_sphere(center, radius, segments=64, rings=32):
    """UV sphere with outward winding and smooth normals: 2*segments + 2*segments*(rings-2) triangles."""
    c = np.asarray(center, dtype=np.float64)

    def vert(i, j):
        th = math.pi * i / rings
        ph = 2.0 * math.pi * (j % segments) / segments
        d = np.array([math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph)])
        return c + radius * d, d

    tris, nrms = [], []

    def add(a, b, cc):
        (pa, na), (pb, nb), (pc, nc) = a, b, cc
        t = np.array([pa, pb, pc])
        if np.dot(np.cross(pb - pa, pc - pa), (pa + pb + pc) / 3.0 - c) < 0:
            t = t[::-1]
            nn = np.array([nc, nb, na])
        else:
            nn = np.array([na, nb, nc])
        tris.append(t)
        nrms.append(nn)

    for j in range(segments):
        add(vert(0, j), vert(1, j), vert(1, j + 1))
        add(vert(rings, j), vert(rings - 1, j + 1), vert(rings - 1, j))
        for i in range(1, rings - 1):
            add(vert(i, j), vert(i + 1, j), vert(i + 1, j + 1))
            add(vert(i, j), vert(i + 1, j + 1), vert(i, j + 1))
    return np.array(tris), np.array(nrms)


def cornell_box(segments: int = 64, rings: int = 32) -> SceneSpec:
    mats = [
        MaterialSpec("white", BRDF_MATTE, (0.73, 0.73, 0.73)),
        MaterialSpec("red", BRDF_MATTE, (0.63, 0.06, 0.05)),
        MaterialSpec("green", BRDF_MATTE, (0.14, 0.45, 0.09)),
        MaterialSpec("light", BRDF_LIGHT, (15.0, 15.0, 15.0)),
        MaterialSpec("mirror", BRDF_MIRROR, (0.95, 0.95, 0.95)),
        MaterialSpec("diffuse", BRDF_MATTE, (0.73, 0.73, 0.73)),
    ]
    parts = []
    P = lambda x, y, z: np.array([x, y, z], dtype=np.float64)
    parts.append((*_quad(P(0, 0, 0), P(1, 0, 0), P(1, 0, 1), P(0, 0, 1), (0, 1, 0)), 0))    # floor
    parts.append((*_quad(P(0, 1, 0), P(1, 1, 0), P(1, 1, 1), P(0, 1, 1), (0, -1, 0)), 0))   # ceiling
    parts.append((*_quad(P(0, 0, 0), P(1, 0, 0), P(1, 1, 0), P(0, 1, 0), (0, 0, 1)), 0))    # back wall
    parts.append((*_quad(P(0, 0, 0), P(0, 1, 0), P(0, 1, 1), P(0, 0, 1), (1, 0, 0)), 1))    # left, red
    parts.append((*_quad(P(1, 0, 0), P(1, 1, 0), P(1, 1, 1), P(1, 0, 1), (-1, 0, 0)), 2))   # right, green
    y = 0.999
    parts.append((*_quad(P(0.375, y, 0.375), P(0.625, y, 0.375), P(0.625, y, 0.625), P(0.375, y, 0.625),
                         (0, -1, 0)), 3))                                                    # light
    st, sn = uv_sphere((0.28, 0.18, 0.30), 0.18, segments, rings)
    parts.append((st, sn, 4))
    dt, dn = uv_sphere((0.72, 0.18, 0.62), 0.18, segments, rings)
    parts.append((dt, dn, 5))
    pos = np.concatenate([p[0] for p in parts]).astype(np.float32)
    nrm = np.concatenate([p[1] for p in parts]).astype(np.float32)
    mid = np.concatenate([np.full(len(p[0]), p[2], dtype=np.int32) for p in parts])
    return SceneSpec(pos, nrm, mid, mats)
