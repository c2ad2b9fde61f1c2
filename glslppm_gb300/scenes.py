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
# the other classes of the reference's material classifier (mesh.cpp:520-611)
BRDF_GLASS, BRDF_PLASTIC, BRDF_GLOSSY, BRDF_GLOSSY_GLASS, BRDF_GLOSSY_PLASTIC = 2, 3, 4, 5, 6


def packed_glossiness(specularity: float) -> float:
    """g = 1 / ((2 / (1 - specularity))^2.71828 + 1) (gpurt.cpp:126), in single precision."""
    f = np.float32
    return float(f(1.0) / (f(f(2.0) / (f(1.0) - f(specularity))) ** f(2.71828) + f(1.0)))


@dataclass
class MaterialSpec:
    name: str
    brdf: int
    color: tuple  # final albedo / emission as the renderer uses it
    eta: float = 1.7
    glossiness: float = 0.0
    specularity: float = 1.0  # Ns / 100 of the glossy classes (>= 0.5), for the MTL block
    texture: np.ndarray | None = None  # map_Kd image, uint8 [h, w, 3], rows top to bottom

    def mtl(self, texture_file: str | None = None) -> str:
        """MTL block that the reference loader classifies into this material (mesh.cpp:520-611):
        Ka > 0 makes a light; Ns = 100 with Ks = (1,1,1) a mirror, with 0 < |Ks|^2 < 3 plastic;
        Ns < 100 the glossy classes; a name starting with "glass" glass, eta = |Ks|^2 / 3 + 1; the
        loader scales matte and plastic albedo by 0.9 and takes the square root of glass albedo."""
        zero = (0.0, 0.0, 0.0)
        ks_eta = (math.sqrt(max(self.eta - 1.0, 0.0)),) * 3  # |Ks|^2 / 3 + 1 = eta
        ns = 100.0 if self.brdf in (BRDF_MIRROR, BRDF_GLASS, BRDF_PLASTIC, BRDF_MATTE) else 100.0 * self.specularity
        if self.brdf == BRDF_LIGHT:
            ka, kd, ks, ns = (1.0, 1.0, 1.0), self.color, zero, 0.0
        elif self.brdf == BRDF_MIRROR:
            ka, kd, ks = zero, self.color, (1.0, 1.0, 1.0)
        elif self.brdf == BRDF_GLOSSY:
            ka, kd, ks = zero, self.color, (1.0, 1.0, 1.0)
        elif self.brdf in (BRDF_GLASS, BRDF_GLOSSY_GLASS):
            if not self.name.startswith("glass"):
                raise ValueError("the reference loader makes glass of materials named glass*")
            ka, kd, ks = zero, tuple(c * c for c in self.color), ks_eta
        elif self.brdf == BRDF_PLASTIC:
            ka, kd, ks = zero, tuple(c / 0.9 for c in self.color), (0.5, 0.5, 0.5)
        elif self.brdf == BRDF_GLOSSY_PLASTIC:
            ka, kd, ks = zero, self.color, (0.5, 0.5, 0.5)
        else:  # matte: the loader scales Lambertian albedo by 0.9
            ka, kd, ks = zero, tuple(c / 0.9 for c in self.color), zero
        f = lambda v: " ".join("%.9g" % x for x in v)
        block = f"newmtl {self.name}\nKa {f(ka)}\nKd {f(kd)}\nKs {f(ks)}\nNs {ns:.1f}\n"
        # the reference gives a map_Kd texture to the material its Ns line completed (mesh.cpp:117-123)
        return block + (f"map_Kd {texture_file}\n" if texture_file else "")


@dataclass
class SceneSpec:
    positions: np.ndarray  # [n, 3, 3] float32
    normals: np.ndarray  # [n, 3, 3] float32
    material_ids: np.ndarray  # [n] int32
    materials: list = field(default_factory=list)
    camera_origin: tuple = (0.5, 0.5, 2.15)
    camera_lookat: tuple = (0.5, 0.5, 0.0)
    fov: float = 45.0
    texcoords: np.ndarray | None = None  # [n, 3, 2] float32 (used by textured materials)

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
        """OBJ + MTL (same stem) in the dialect of the reference loader; textures as binary PPM
        files beside them (<stem>_<material index>.ppm)."""
        path = Path(path)
        mtl = path.with_suffix(".mtl")
        blocks = []
        for k, m in enumerate(self.materials):
            tex_name = None
            if m.texture is not None:
                tex_name = f"{path.stem}_{k}.ppm"
                img = np.ascontiguousarray(m.texture, dtype=np.uint8)
                (path.parent / tex_name).write_bytes(b"P6\n%d %d\n255\n" % (img.shape[1], img.shape[0]) + img.tobytes())
            blocks.append(m.mtl(tex_name) + "\n")
        mtl.write_text("".join(blocks))
        lines = [f"mtllib {mtl.name}\n"]
        n = self.num_triangles
        p = self.positions.reshape(-1, 3)
        nr = self.normals.reshape(-1, 3)
        lines += ["v %.9g %.9g %.9g\n" % tuple(map(float, v)) for v in p]
        lines += ["vn %.9g %.9g %.9g\n" % tuple(map(float, v)) for v in nr]
        if self.texcoords is not None:
            lines += ["vt %.9g %.9g\n" % tuple(map(float, v)) for v in self.texcoords.reshape(-1, 2)]
        cur = None
        for t in range(n):
            m = int(self.material_ids[t])
            if m != cur:
                lines.append(f"usemtl {self.materials[m].name}\n")
                cur = m
            a, b, c = 3 * t + 1, 3 * t + 2, 3 * t + 3
            if self.texcoords is not None:
                lines.append(f"f {a}/{a}/{a} {b}/{b}/{b} {c}/{c}/{c}\n")
            else:
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
    """UV sphere with outward winding and smooth normals: 2*segments + 2*segments*(rings-2) triangles.

    Triangle order, per segment j: the north cap (0,j)(1,j)(1,j+1), the south cap
    (R,j)(R-1,j+1)(R-1,j), then rings 1..R-2 as two triangles each; a triangle whose winding
    faces inwards is reversed (vertices and normals)."""
    c = np.asarray(center, dtype=np.float64)
    # unit directions of the (rings+1) x segments vertex grid (the trigonometry of Python's math)
    d = np.empty((rings + 1, segments, 3), dtype=np.float64)
    for i in range(rings + 1):
        th = math.pi * i / rings
        st, ct = math.sin(th), math.cos(th)
        for j in range(segments):
            ph = 2.0 * math.pi * j / segments
            d[i, j] = (st * math.cos(ph), ct, st * math.sin(ph))
    p = c + radius * d
    # per segment: the two caps, then rings 1..R-2 as two triangles each; (ring, segment) pairs
    nr = rings - 2
    jj = np.arange(segments)[:, None]
    jn = (jj + 1) % segments
    i = np.arange(1, rings - 1)[None, :]
    idx = np.empty((segments, 2 + 2 * nr, 3, 2), dtype=np.int64)
    idx[:, 0] = np.stack([np.stack([np.zeros_like(jj[:, 0]), jj[:, 0]], -1),
                          np.stack([np.ones_like(jj[:, 0]), jj[:, 0]], -1),
                          np.stack([np.ones_like(jj[:, 0]), jn[:, 0]], -1)], 1)
    idx[:, 1] = np.stack([np.stack([np.full_like(jj[:, 0], rings), jj[:, 0]], -1),
                          np.stack([np.full_like(jj[:, 0], rings - 1), jn[:, 0]], -1),
                          np.stack([np.full_like(jj[:, 0], rings - 1), jj[:, 0]], -1)], 1)
    if nr > 0:
        I, J, JN = np.broadcast_arrays(i, jj, jn)
        a = np.stack([np.stack([I, J], -1), np.stack([I + 1, J], -1), np.stack([I + 1, JN], -1)], 2)
        b = np.stack([np.stack([I, J], -1), np.stack([I + 1, JN], -1), np.stack([I, JN], -1)], 2)
        idx[:, 2::2] = a
        idx[:, 3::2] = b
    idx = idx.reshape(-1, 3, 2)
    tris = p[idx[..., 0], idx[..., 1]]
    nrms = d[idx[..., 0], idx[..., 1]]
    cen = (tris[:, 0] + tris[:, 1] + tris[:, 2]) / 3.0
    face = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    flip = np.einsum("ij,ij->i", face, cen - c) < 0
    tris[flip] = tris[flip][:, ::-1]
    nrms[flip] = nrms[flip][:, ::-1]
    return tris, nrms


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


def materials_box(segments: int = 16, rings: int = 8, light: bool = True) -> SceneSpec:
    """The Cornell box with a material of every class the reference's classifier makes: the two
    spheres are half glass / half glossy glass and half plastic / half glossy plastic, the left
    wall glossy metal.  light=False turns the ceiling light into a white wall: with no emitting
    triangle the photons come from the environment (GenerateIBLSample, photontrace.fs:283-341)
    and eye rays that leave the scene see the sky colour."""
    sc = cornell_box(segments, rings)
    mats = list(sc.materials) + [
        MaterialSpec("glass", BRDF_GLASS, (0.95, 0.95, 0.95), eta=1.5),
        MaterialSpec("plastic", BRDF_PLASTIC, (0.6, 0.3, 0.2)),
        MaterialSpec("glossy", BRDF_GLOSSY, (0.8, 0.8, 0.8), glossiness=packed_glossiness(0.5), specularity=0.5),
        MaterialSpec("glass_glossy", BRDF_GLOSSY_GLASS, (0.9, 0.9, 0.95), eta=1.5,
                     glossiness=packed_glossiness(0.6), specularity=0.6),
        MaterialSpec("plastic_glossy", BRDF_GLOSSY_PLASTIC, (0.2, 0.5, 0.7), glossiness=packed_glossiness(0.7),
                     specularity=0.7),
    ]
    ids = sc.material_ids.copy()
    s1, s2 = np.nonzero(ids == 4)[0], np.nonzero(ids == 5)[0]
    ids[s1[: len(s1) // 2]], ids[s1[len(s1) // 2:]] = 6, 9
    ids[s2[: len(s2) // 2]], ids[s2[len(s2) // 2:]] = 7, 10
    ids[ids == 1] = 8
    if not light:
        ids[ids == 3] = 0
    return SceneSpec(sc.positions, sc.normals, ids, mats, sc.camera_origin, sc.camera_lookat, sc.fov)


def textured_box(segments: int = 16, rings: int = 8) -> SceneSpec:
    """The Cornell box with map_Kd textures (the reference's VolumeTextureTextures): a checker on
    the white walls, a 53x37 gradient on the green wall (not a power of two: the reference's
    nearest resampling to 512x512), a textured light and striped diffuse sphere; planar texture
    coordinates that run past 1 (GL_REPEAT).  Load it through write_obj + Mesh.load_obj (the
    from-arrays path carries no textures)."""
    import dataclasses
    sc = cornell_box(segments, rings)
    yy, xx = np.mgrid[0:64, 0:64]
    on = ((xx // 8) + (yy // 8)) % 2 == 0
    checker = np.stack([np.where(on, 230, 40), np.full_like(xx, 180), np.where(on, 30, 220)], -1).astype(np.uint8)
    gy, gx = np.mgrid[0:37, 0:53]
    gradient = np.stack([gx * 255 // 52, gy * 255 // 36, np.full_like(gx, 128)], -1).astype(np.uint8)
    glow = np.random.default_rng(11).integers(150, 256, size=(16, 16, 3)).astype(np.uint8)
    sy, sx = np.mgrid[0:32, 0:128]
    stripes = np.stack([np.where((sx // 16) % 2 == 0, 250, 60), np.full_like(sx, 90), np.full_like(sx, 200)],
                       -1).astype(np.uint8)
    mats = [dataclasses.replace(m) for m in sc.materials]
    for k, tex in ((0, checker), (2, gradient), (3, glow), (5, stripes)):
        mats[k] = dataclasses.replace(mats[k], texture=tex)
    p = sc.positions.astype(np.float64)
    uv = np.stack([2.0 * p[..., 0] + 0.37 * p[..., 1], 2.0 * p[..., 2] - 0.53 * p[..., 1]], -1).astype(np.float32)
    return SceneSpec(sc.positions, sc.normals, sc.material_ids, mats, sc.camera_origin, sc.camera_lookat, sc.fov,
                     texcoords=uv)


@dataclass
class JobSpec:
    """One job of the batched workload: a scene and its image / photon sizes."""
    scene: SceneSpec
    width: int
    height: int
    photon_width: int
    photon_height: int
    seed: int


def _box(lo, hi):
    """axis-aligned box as 12 outward-facing triangles with flat normals"""
    lo, hi = np.asarray(lo, dtype=np.float64), np.asarray(hi, dtype=np.float64)
    P = lambda x, y, z: np.array([[lo, hi][x][0], [lo, hi][y][1], [lo, hi][z][2]])
    faces = [((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, -1, 0)),
             ((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1), (0, 1, 0)),
             ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, -1)),
             ((0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1), (0, 0, 1)),
             ((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (-1, 0, 0)),
             ((1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1), (1, 0, 0))]
    tris, nrms = [], []
    for a, b, c, d, n in faces:
        t, nn = _quad(P(*a), P(*b), P(*c), P(*d), n)
        tris.append(t)
        nrms.append(nn)
    return np.concatenate(tris), np.concatenate(nrms)


def cornell_variant(seed: int, min_tris: int = 10_000, max_tris: int = 500_000) -> JobSpec:
    """A procedurally generated Cornell box of the batched workload: the five walls and ceiling
    light of cornell_box() plus 1-40 random spheres and boxes, with a triangle count drawn
    log-uniformly from [min_tris, max_tris] (spread over the spheres' tessellation), an image of
    128^2, 256^2, 512^2 or 1024^2 pixels and 2^14 .. 2^19 photon slots per pass (a 2^(e/2)
    square, or 2^((e+1)/2) x 2^((e-1)/2) for odd e).  Materials: Lambertian albedo uniform in
    [0.2, 0.8] (75 %), mirror (15 %), glass of index 1.5 (10 %)."""
    rng = np.random.default_rng(0x5eed0000 + seed)
    base = cornell_box(segments=8, rings=4)
    keep = base.material_ids <= 3  # walls and light
    pos, nrm, mid = [base.positions[keep]], [base.normals[keep]], [base.material_ids[keep]]
    mats = list(base.materials[:4])
    target = int(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris))))
    n_obj = int(rng.integers(1, 41))
    kinds = rng.random(n_obj) < 0.7  # True: sphere
    if not kinds.any():
        kinds[0] = True
    n_sph = int(kinds.sum())
    budget = max(target - 12 * (n_obj - n_sph) - 12, 64)
    seg = max(8, int(math.sqrt(budget / n_sph)) // 2 * 2)
    for k in range(n_obj):
        u = rng.random()
        if u < 0.75:
            alb = tuple(float(x) for x in rng.uniform(0.2, 0.8, 3))
            mats.append(MaterialSpec(f"m{k}", BRDF_MATTE, alb))
        elif u < 0.9:
            mats.append(MaterialSpec(f"m{k}", BRDF_MIRROR, (0.95, 0.95, 0.95)))
        else:
            mats.append(MaterialSpec(f"m{k}", 2, (0.98, 0.98, 0.98), eta=1.5))
        m = len(mats) - 1
        if kinds[k]:
            r = float(rng.uniform(0.03, 0.15))
            c = (rng.uniform(r, 1 - r), rng.uniform(r, 0.9 - r), rng.uniform(r, 1 - r))
            t, n = uv_sphere(c, r, seg, seg // 2)
        else:
            h = rng.uniform(0.03, 0.15, 3)
            c = np.array([rng.uniform(h[0], 1 - h[0]), rng.uniform(h[1], 0.9 - h[1]), rng.uniform(h[2], 1 - h[2])])
            t, n = _box(c - h, c + h)
        pos.append(t.astype(np.float32))
        nrm.append(n.astype(np.float32))
        mid.append(np.full(len(t), m, dtype=np.int32))
    sc = SceneSpec(np.concatenate(pos), np.concatenate(nrm), np.concatenate(mid), mats)
    res = int(rng.choice([128, 256, 512, 1024]))
    e = int(rng.integers(14, 20))
    return JobSpec(sc, res, res, 1 << ((e + 1) // 2), 1 << (e // 2), seed)


def perlin(p: np.ndarray, seed: int) -> np.ndarray:
    """Classic gradient noise (Perlin 2002: quintic fade, 12 edge gradients, a seeded permutation
    of 256) at the points p [..., 3]; values roughly in [-1, 1]."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    perm = np.concatenate([perm, perm]).astype(np.int64)
    grad = np.array([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
                     [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], dtype=np.float64)
    p = np.asarray(p, dtype=np.float64)
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    pi &= 255
    fade = pf * pf * pf * (pf * (pf * 6 - 15) + 10)
    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                h = perm[perm[perm[pi[..., 0] + dx] + pi[..., 1] + dy] + pi[..., 2] + dz] % 12
                g = grad[h]
                d = pf - np.array([dx, dy, dz], dtype=np.float64)
                w = np.where(dx, fade[..., 0], 1 - fade[..., 0]) * np.where(dy, fade[..., 1], 1 - fade[..., 1]) * \
                    np.where(dz, fade[..., 2], 1 - fade[..., 2])
                out = out + w * np.einsum("...k,...k->...", g, d)
    return out


def _face_normals(tris: np.ndarray) -> np.ndarray:
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return np.repeat(n[:, None, :], 3, axis=1)


def geodesic_sphere(center, radius, freq: int, displace, seed: int):
    """Icosahedron with every face split into freq^2 triangles, projected to the sphere and
    displaced radially by radius * displace * noise(3 * direction): 20 * freq^2 triangles."""
    t = (1 + 5 ** 0.5) / 2
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    m = freq
    i, j = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    up = (i + j) < m
    dn = (i + j) < m - 1
    ui, uj = i[up], j[up]
    di, dj = i[dn], j[dn]
    # barycentric (a, b) of the lattice points of one face, per triangle corner
    up_ab = np.stack([np.stack([ui, uj], -1), np.stack([ui + 1, uj], -1), np.stack([ui, uj + 1], -1)], 1)
    dn_ab = np.stack([np.stack([di + 1, dj], -1), np.stack([di + 1, dj + 1], -1), np.stack([di, dj + 1], -1)], 1)
    ab = np.concatenate([up_ab, dn_ab]).astype(np.float64) / m  # [m^2, 3, 2]
    A, B, Cc = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]  # [20, 3]
    pts = (A[:, None, None, :] + ab[None, ..., 0:1] * (B - A)[:, None, None, :] +
           ab[None, ..., 1:2] * (Cc - A)[:, None, None, :]).reshape(-1, 3, 3)
    d = pts / np.linalg.norm(pts, axis=-1, keepdims=True)
    r = radius * (1.0 + displace * perlin(3.0 * d + 17.0, seed))
    tris = np.asarray(center, dtype=np.float64) + d * r[..., None]
    # outward winding
    cen = tris.mean(1) - np.asarray(center)
    fn = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    flip = np.einsum("ij,ij->i", fn, cen) < 0
    tris[flip] = tris[flip][:, ::-1]
    return tris


def heightfield(size: float, verts: int, height: float, seed: int):
    """A verts x verts grid over [-size, size]^2 at y = height * noise: 2 (verts-1)^2 triangles."""
    x = np.linspace(-size, size, verts)
    X, Z = np.meshgrid(x, x, indexing="ij")
    Y = height * perlin(np.stack([X * 3.0, np.full_like(X, 0.5), Z * 3.0], -1), seed + 1)
    P = np.stack([X, Y, Z], -1)
    a, b, c, d = P[:-1, :-1], P[1:, :-1], P[1:, 1:], P[:-1, 1:]
    t1 = np.stack([a, d, c], 2).reshape(-1, 3, 3)  # y-up winding
    t2 = np.stack([a, c, b], 2).reshape(-1, 3, 3)
    return np.concatenate([t1, t2])


def large_mesh(seed: int = 1, sphere_freq: int = 317, floor_verts: int = 1024, n_albedo: int = 4000) -> SceneSpec:
    """The large-mesh workload: a Perlin-displaced geodesic sphere (20 * 317^2 = 2.01M triangles)
    on a Perlin heightfield floor of 1024 x 1024 vertices (2.09M triangles), per-triangle albedo
    uniform in [0.2, 0.8] quantised to 4000 materials, 10% of the triangles mirrors, and four
    random quad area lights of emission 5-20 above the scene."""
    rng = np.random.default_rng(0x1a46e000 + seed)
    sph = geodesic_sphere((0.0, 0.75, 0.0), 0.6, sphere_freq, 0.08, seed)
    flo = heightfield(2.0, floor_verts, 0.1, seed)
    geo = np.concatenate([sph, flo])
    n = len(geo)
    alb = rng.uniform(0.2, 0.8, size=(n_albedo, 3))
    mats = [MaterialSpec(f"a{k}", BRDF_MATTE, tuple(float(c) for c in alb[k])) for k in range(n_albedo)]
    mats.append(MaterialSpec("mirror", BRDF_MIRROR, (0.95, 0.95, 0.95)))
    mid = rng.integers(0, n_albedo, n).astype(np.int32)
    mid[rng.random(n) < 0.1] = n_albedo
    lights = []
    for k in range(4):
        e = float(rng.uniform(5.0, 20.0))
        mats.append(MaterialSpec(f"light{k}", BRDF_LIGHT, (e, e, e)))
        cx, cz = rng.uniform(-1.2, 1.2, 2)
        h = float(rng.uniform(0.15, 0.3))
        y = float(rng.uniform(2.0, 2.6))
        t, _ = _quad(np.array([cx - h, y, cz - h]), np.array([cx + h, y, cz - h]), np.array([cx + h, y, cz + h]),
                     np.array([cx - h, y, cz + h]), (0, -1, 0))
        lights.append((t, len(mats) - 1))
    ltris = np.concatenate([t for t, _ in lights])
    lmid = np.concatenate([np.full(2, m, dtype=np.int32) for _, m in lights])
    pos = np.concatenate([geo, ltris]).astype(np.float32)
    mid = np.concatenate([mid, lmid])
    return SceneSpec(pos, _face_normals(pos.astype(np.float64)).astype(np.float32), mid, mats,
                     camera_origin=(0.0, 1.6, 3.2), camera_lookat=(0.0, 0.6, 0.0), fov=45.0)
