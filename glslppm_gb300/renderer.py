"""Host-side mirror of the reference's interface for the SPPM path.

``Mesh`` plays the part of ``TMesh`` + ``TBVH`` (mesh.cpp, bvh.cpp): OBJ/MTL loading or flat
arrays, and the six threaded BVH orderings.  ``Renderer`` plays the part of ``CGPURT``
(gpurt.h:29-67) together with the frame driver ``m_display`` (glslppm.cpp:214-536): upload the
scene (``precalculate_mesh_data``), set the camera, run SPPM frames (``display``), read the image
(``re.fs``) and any state texture.  Every call goes through the C ABI of ``libsppm.so``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import native as N


def _fptr(a: np.ndarray, ctype=C.c_float):
    return a.ctypes.data_as(C.POINTER(ctype))


def default_config(resolution: int = 512, **overrides) -> N.Config:
    """The reference's constants (glslppm.cpp:28-40, 488) for a square image; keyword overrides."""
    cfg = N.Config()
    N.lib.sppm_config_defaults(C.byref(cfg), resolution)
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise AttributeError(f"sppm_config has no field {k!r}")
        setattr(cfg, k, v)
    return cfg


def look_at(origin, lookat, width: int, height: int, fov_degrees: float = 45.0) -> N.Camera:
    """TCamera::Set (camera.cpp:4-18)."""
    cam = N.Camera()
    o = (C.c_float * 3)(*origin)
    l = (C.c_float * 3)(*lookat)
    N.lib.sppm_camera_look_at(C.byref(cam), o, l, width, height, C.c_float(fov_degrees))
    return cam


@dataclass
class SceneArrays:
    """Copies of the arrays an sppm_scene points to (for tests and fixtures)."""

    positions: np.ndarray
    normals: np.ndarray
    texcoords: np.ndarray
    material_ids: np.ndarray
    materials: np.ndarray  # structured: color[3], eta, brdf, glossiness
    light_triangles: np.ndarray
    light_cdf: np.ndarray
    light_area: float
    bbox_min: np.ndarray
    bbox_max: np.ndarray
    node_bounds: np.ndarray
    node_triangle: np.ndarray
    order_base: np.ndarray
    order_miss: np.ndarray
    # material textures: [num_textures, 512, 512, 4] uint8 and [num_materials] layer or -1
    textures: np.ndarray = field(default_factory=lambda: np.zeros((0, 512, 512, 4), np.uint8))
    material_texture: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))


MATERIAL_DTYPE = np.dtype([("color", "<f4", 3), ("eta", "<f4"), ("brdf", "<i4"), ("glossiness", "<f4")])


class Mesh:
    """An sppm_mesh: triangles, materials, light table and (after build_bvh) the BVH."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def load_obj(cls, path: str, offset=(0.0, 0.0, 0.0), scale: float = 1.0) -> "Mesh":
        out = C.c_void_p()
        off = (C.c_float * 3)(*offset)
        N.check(N.lib.sppm_mesh_load_obj(str(path).encode(), off, C.c_float(scale), C.byref(out)))
        return cls(out.value)

    @classmethod
    def from_arrays(cls, positions, material_ids, materials, normals=None) -> "Mesh":
        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 9)
        mid = np.ascontiguousarray(material_ids, dtype=np.int32).reshape(-1)
        mats = np.ascontiguousarray(materials, dtype=MATERIAL_DTYPE)
        nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 9)
        if len(mid) != len(pos):
            raise ValueError("one material id per triangle")
        out = C.c_void_p()
        N.check(N.lib.sppm_mesh_from_arrays(len(pos), pos.ctypes.data, None if nrm is None else nrm.ctypes.data,
                                            mid.ctypes.data, len(mats), mats.ctypes.data, C.byref(out)))
        return cls(out.value)

    def build_bvh(self, gpu: bool = False, device: int = 0, builder: str = "ploc") -> "Mesh":
        """TBVH::Build on the host (the reference's exact-SAH tree), or with gpu=True the same
        arrays from a tree built on the GPU (a different tree, milliseconds per million triangles):
        builder "ploc" (locally-ordered clustering, near-SAH quality) or "lbvh" (radix tree)."""
        if gpu:
            b = {"ploc": N.BVH_GPU_PLOC, "lbvh": N.BVH_GPU_LBVH}[builder]
            N.check(N.lib.sppm_mesh_build_bvh_gpu_ex(self._h, device, b))
        else:
            N.check(N.lib.sppm_mesh_build_bvh(self._h))
        return self

    def scene(self) -> N.Scene:
        s = N.Scene()
        N.check(N.lib.sppm_mesh_get_scene(self._h, C.byref(s)))
        s._owner = self  # keep the mesh alive while the struct is in use
        return s

    def arrays(self) -> SceneArrays:
        s = self.scene()
        n, nn, nm, nl = s.num_triangles, s.num_nodes, s.num_materials, s.num_lights

        def grab(ptr, count, dtype):
            if count == 0 or not ptr:
                return np.zeros(0, dtype=dtype)
            return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dtype).copy()

        mats = np.zeros(nm, dtype=MATERIAL_DTYPE)
        C.memmove(mats.ctypes.data, s.materials, nm * MATERIAL_DTYPE.itemsize)
        return SceneArrays(
            positions=grab(s.positions, n * 9, np.float32).reshape(n, 3, 3),
            normals=grab(s.normals, n * 9, np.float32).reshape(n, 3, 3),
            texcoords=grab(s.texcoords, n * 6, np.float32).reshape(n, 3, 2),
            material_ids=grab(s.material_ids, n, np.int32),
            materials=mats,
            light_triangles=grab(s.light_triangles, nl, np.int32),
            light_cdf=grab(s.light_cdf, nl, np.float32),
            light_area=float(s.light_area),
            bbox_min=np.array(list(s.bbox_min), dtype=np.float32),
            bbox_max=np.array(list(s.bbox_max), dtype=np.float32),
            node_bounds=grab(s.node_bounds, nn * 6, np.float32).reshape(nn, 6),
            node_triangle=grab(s.node_triangle, nn, np.int32),
            order_base=grab(s.order_base, nn * 6, np.int32).reshape(6, nn),
            order_miss=grab(s.order_miss, nn * 6, np.int32).reshape(6, nn),
            textures=grab(s.textures, s.num_textures * 512 * 512 * 4, np.uint8).reshape(-1, 512, 512, 4),
            material_texture=grab(s.material_texture, nm if s.material_texture else 0, np.int32),
        )

    @property
    def num_triangles(self) -> int:
        return int(self.scene().num_triangles)

    def close(self) -> None:
        if self._h and self._h.value:
            N.lib.sppm_mesh_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def scene_from_arrays(a: SceneArrays) -> N.Scene:
    """An sppm_scene pointing at numpy arrays (kept alive by the returned struct)."""
    keep = {}

    def arr(x, dtype):
        x = np.ascontiguousarray(x, dtype=dtype)
        keep[id(x)] = x
        return x

    s = N.Scene()
    pos = arr(a.positions, np.float32)
    s.num_triangles = pos.shape[0]
    s.positions = _fptr(pos)
    s.normals = _fptr(arr(a.normals, np.float32))
    s.texcoords = _fptr(arr(a.texcoords, np.float32))
    s.material_ids = _fptr(arr(a.material_ids, np.int32), C.c_int32)
    mats = arr(a.materials, MATERIAL_DTYPE)
    s.num_materials = len(mats)
    s.materials = C.cast(mats.ctypes.data, C.POINTER(N.Material))
    lt = arr(a.light_triangles, np.int32)
    s.num_lights = len(lt)
    s.light_triangles = _fptr(lt, C.c_int32)
    s.light_cdf = _fptr(arr(a.light_cdf, np.float32))
    s.light_area = float(a.light_area)
    for k in range(3):
        s.bbox_min[k] = float(a.bbox_min[k])
        s.bbox_max[k] = float(a.bbox_max[k])
    nb = arr(a.node_bounds, np.float32)
    s.num_nodes = nb.shape[0]
    s.node_bounds = _fptr(nb)
    s.node_triangle = _fptr(arr(a.node_triangle, np.int32), C.c_int32)
    s.order_base = _fptr(arr(a.order_base, np.int32), C.c_int32)
    s.order_miss = _fptr(arr(a.order_miss, np.int32), C.c_int32)
    tex = arr(getattr(a, "textures", np.zeros((0, 512, 512, 4), np.uint8)), np.uint8)
    s.num_textures = tex.shape[0] if tex.size else 0
    if s.num_textures:
        s.textures = C.cast(tex.ctypes.data, C.POINTER(C.c_uint8))
        s.material_texture = _fptr(arr(a.material_texture, np.int32), C.c_int32)
    s._keep = keep
    return s


def _state_array(kind: str, nbytes: int) -> np.ndarray:
    """An empty host array of the element type and shape of a state kind."""
    if kind in ("hit_triangle",):
        return np.empty(nbytes // 4, dtype=np.int32)
    if kind in ("slot_winner", "slot_count"):
        return np.empty(nbytes // 4, dtype=np.uint32)
    if kind == "photon_hit":
        return np.empty((nbytes // 8, 2), dtype=np.int32)
    if kind == "hit_t":
        return np.empty(nbytes // 4, dtype=np.float32)
    if kind.startswith("stats_"):
        return np.empty(nbytes // 8, dtype=np.float64)
    return np.empty((nbytes // 16, 4), dtype=np.float32)


def _check_image_buffer(out: np.ndarray, width: int, height: int) -> None:
    if (not isinstance(out, np.ndarray) or out.dtype != np.float32 or not out.flags.c_contiguous
            or out.size != width * height * 3):
        raise N.SppmError(N.ERR_ARG, f"image buffer must be C-contiguous float32 with {width * height * 3} elements")


def _release_tickets(inflight: dict, ticket: int) -> None:
    for t in [t for t in inflight if t <= ticket]:
        del inflight[t]


class Renderer:
    """One SPPM render job on one GPU (CGPURT + m_display)."""

    def __init__(self, config: N.Config, device: int = 0):
        self.config = config
        out = C.c_void_p()
        N.check(N.lib.sppm_create(C.byref(config), device, C.byref(out)))
        self._h = out
        self.width, self.height = config.width, config.height
        self._inflight: dict[int, np.ndarray] = {}  # host images of copies not yet waited for

    # CGPURT::PrecalculateMeshData + CreateTextures
    def upload_scene(self, scene) -> None:
        if isinstance(scene, Mesh):
            scene = scene.scene()
        elif isinstance(scene, SceneArrays):
            scene = scene_from_arrays(scene)
        N.check(N.lib.sppm_upload_scene(self._h, C.byref(scene)))

    precalculate_mesh_data = upload_scene

    def set_camera(self, cam: N.Camera) -> None:
        N.check(N.lib.sppm_set_camera(self._h, C.byref(cam)))

    def reset(self) -> None:
        N.check(N.lib.sppm_reset(self._h))

    def run_passes(self, n: int = 1) -> None:
        N.check(N.lib.sppm_run_passes(self._h, n))

    def display(self) -> None:
        """One SPPM frame (m_display)."""
        self.run_passes(1)

    def synchronize(self) -> None:
        N.check(N.lib.sppm_synchronize(self._h))
        self._inflight.clear()

    def read_image(self, kind: int = N.IMAGE_RADIANCE, out: np.ndarray | None = None) -> np.ndarray:
        n = self.width * self.height * 3
        if out is None:
            out = np.empty((self.height, self.width, 3), dtype=np.float32)
        N.check(N.lib.sppm_read_image(self._h, kind, out.ctypes.data, n))
        return out

    def read_image_async(self, out: np.ndarray, kind: int = N.IMAGE_RADIANCE) -> int:
        """Queues the resolve and the copy into `out` (page-locked, e.g. pinned_empty, for the
        copy to overlap the next passes) and returns its ticket; `out` holds the image once
        image_wait(ticket) or synchronize() has returned."""
        _check_image_buffer(out, self.width, self.height)
        t = C.c_uint64()
        N.check(N.lib.sppm_read_image_async(self._h, kind, out.ctypes.data, out.size, C.byref(t)))
        self._inflight[int(t.value)] = out
        return int(t.value)

    def image_wait(self, ticket: int) -> None:
        N.check(N.lib.sppm_image_wait(self._h, ticket))
        _release_tickets(self._inflight, ticket)

    def image_done(self, ticket: int) -> bool:
        done = C.c_int()
        N.check(N.lib.sppm_image_query(self._h, ticket, C.byref(done)))
        if done.value:
            _release_tickets(self._inflight, ticket)
        return bool(done.value)

    def state_bytes(self, kind: str) -> int:
        return int(N.lib.sppm_state_bytes(self._h, N.STATE[kind]))

    def read_state(self, kind: str) -> np.ndarray:
        k = N.STATE[kind]
        nbytes = self.state_bytes(kind)
        if nbytes == 0:
            raise N.SppmError(N.ERR_ARG, f"state {kind} is not kept by this context")
        out = _state_array(kind, nbytes)
        N.check(N.lib.sppm_read_state(self._h, k, out.ctypes.data, nbytes))
        return out

    def debug_trace(self, org: np.ndarray, dir: np.ndarray, photon: bool = True, cull: bool = False,
                    mode: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """Single rays through the exact traversal of the uploaded scene: (triangle or -1, t).
        mode 0 traces one ray per thread, mode 1 one ray per warp, mode 2 one ray per block; mode 3
        the mixed path's 4-wide quantised BVH (mixed-precision contexts)."""
        org = np.ascontiguousarray(org, dtype=np.float32).reshape(-1, 3)
        dir = np.ascontiguousarray(dir, dtype=np.float32).reshape(-1, 3)
        n = org.shape[0]
        tri = np.empty(n, dtype=np.int32)
        t = np.empty(n, dtype=np.float32)
        N.check(N.lib.sppm_debug_trace(self._h, org.ctypes.data, dir.ctypes.data, n, int(photon), int(cull), mode,
                                       tri.ctypes.data, t.ctypes.data))
        return tri, t

    def debug_photon_rays(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """The photon rays the last pass traced: (origins [n, 3], directions [n, 3], photon slots [n])."""
        n = C.c_size_t()
        N.check(N.lib.sppm_debug_photon_rays(self._h, None, None, None, 0, C.byref(n)))
        cnt = n.value
        org = np.empty((cnt, 3), np.float32)
        dir = np.empty((cnt, 3), np.float32)
        ph = np.empty(cnt, np.uint32)
        N.check(N.lib.sppm_debug_photon_rays(self._h, org.ctypes.data, dir.ctypes.data, ph.ctypes.data, cnt,
                                             C.byref(n)))
        return org[: n.value], dir[: n.value], ph[: n.value]

    def debug_ray_bins(self) -> tuple[np.ndarray, np.ndarray]:
        """The photon traversal's bin order (binned contexts): (rank [bins] = each bin's position,
        cost [bins] uint64 per position = (node steps << 32) + rays since the last reorder)."""
        n = C.c_uint32()
        N.check(N.lib.sppm_debug_ray_bins(self._h, None, None, 0, C.byref(n)))
        rank = np.empty(n.value, np.uint32)
        cost = np.empty(n.value, np.uint64)
        N.check(N.lib.sppm_debug_ray_bins(self._h, rank.ctypes.data, cost.ctypes.data, n.value, C.byref(n)))
        return rank, cost

    def debug_photon_grid(self) -> tuple[np.ndarray, np.ndarray]:
        """The counting-sort photon grid of the last pass (SPPM_FLAG_PHOTON_GRID): (offsets
        [hash_slots + 1], records [n, 4] uint32 in slot order; within a slot in no fixed order)."""
        n = C.c_uint32()
        N.check(N.lib.sppm_debug_photon_grid(self._h, None, 0, None, 0, C.byref(n)))
        hn = self.config.hash_slots or self.config.photon_width * self.config.photon_height
        ofs = np.empty(hn + 1, np.uint32)
        rec = np.empty((max(n.value, 1), 4), np.uint32)
        N.check(N.lib.sppm_debug_photon_grid(self._h, ofs.ctypes.data, ofs.size, rec.ctypes.data, rec.size,
                                             C.byref(n)))
        return ofs, rec[: n.value]

    def save_checkpoint(self) -> bytes:
        """The progressive state as a flat binary (sppm_save_checkpoint)."""
        n = int(N.lib.sppm_checkpoint_bytes(self._h))
        buf = C.create_string_buffer(n)
        N.check(N.lib.sppm_save_checkpoint(self._h, buf, n))
        return buf.raw

    def load_checkpoint(self, data: bytes) -> None:
        N.check(N.lib.sppm_load_checkpoint(self._h, data, len(data)))

    def frame_info(self) -> N.FrameInfo:
        fi = N.FrameInfo()
        N.check(N.lib.sppm_get_frame_info(self._h, C.byref(fi)))
        return fi

    def enable_stage_timing(self, enable: bool = True) -> None:
        N.check(N.lib.sppm_enable_stage_timing(self._h, 1 if enable else 0))

    def time_stages(self, stages) -> None:
        """Times only the named stages (see native.STAGES); an empty list turns timing off."""
        mask = 0
        for s in stages:
            mask |= 1 << N.STAGES.index(s)
        N.check(N.lib.sppm_set_stage_timing_mask(self._h, mask))

    def read_stage_times(self) -> dict:
        ms = (C.c_float * len(N.STAGES))()
        n = (C.c_uint32 * len(N.STAGES))()
        N.check(N.lib.sppm_read_stage_times(self._h, ms, n))
        return {name: (float(ms[i]), int(n[i])) for i, name in enumerate(N.STAGES)}

    def traversal_counters(self, passes: int = 10) -> dict:
        """Runs `passes` more frames with the counting photon kernel; returns the mean BVH nodes
        visited and triangles tested per photon segment."""
        f0 = self.frame_info()
        N.check(N.lib.sppm_enable_traversal_counters(self._h, 1))
        try:
            self.run_passes(passes)
            self.synchronize()
        finally:
            N.check(N.lib.sppm_enable_traversal_counters(self._h, 0))
        f1 = self.frame_info()
        segs = f1.counted_segments - f0.counted_segments
        return {"passes": passes, "photon_segments": segs,
                "nodes_per_segment": (f1.counted_nodes - f0.counted_nodes) / max(segs, 1),
                "tris_per_segment": (f1.counted_triangles - f0.counted_triangles) / max(segs, 1)}

    def time_passes(self, n: int) -> float:
        ms = C.c_float()
        N.check(N.lib.sppm_time_passes(self._h, n, C.byref(ms)))
        return float(ms.value)

    def set_tuning(self, tuning=None, **fields) -> None:
        """Launch shapes (sppm_tuning): an N.Tuning, or its fields by name (others 0 = default)."""
        t = tuning if tuning is not None else N.Tuning(**fields)
        N.check(N.lib.sppm_set_tuning(self._h, C.byref(t)))

    def get_tuning(self) -> N.Tuning:
        t = N.Tuning()
        N.check(N.lib.sppm_get_tuning(self._h, C.byref(t)))
        return t

    def autotune(self, cycles: int = 1) -> tuple[N.Tuning, float]:
        """Runs the next passes under candidate launch shapes and keeps the fastest; returns the
        shapes chosen and their device time per pass (ms)."""
        t, ms = N.Tuning(), C.c_float()
        N.check(N.lib.sppm_autotune(self._h, cycles, C.byref(t), C.byref(ms)))
        return t, float(ms.value)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            N.lib.sppm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def hash_build(d_pos: int, d_flux: int, photon_width: int, photon_height: int, hash_slots: int, bbox_min,
               grid_scale: float, flags: int, d_winner: int, d_count: int, stream: int = 0) -> None:
    """Stage-level hashed-grid build on device pointers (sppm_hash_build)."""
    bb = (C.c_float * 3)(*bbox_min)
    N.check(N.lib.sppm_hash_build(d_pos, d_flux, photon_width, photon_height, hash_slots, bb, C.c_float(grid_scale),
                                  flags, d_winner, d_count, stream))


REDUCE_MIN, REDUCE_MAX, REDUCE_SUM = 0, 1, 2


def tune_hash_slots(cfg: N.Config, scene, camera: N.Camera, passes: int = 20, device: int = 0) -> tuple[int, list]:
    """The hash-table size by measurement (sppm_tune_hash_slots): hash_slots of P, 2P and 4P
    photon slots timed in scratch contexts; returns the fastest and the three times per pass (ms;
    -1 for a size that was not a candidate)."""
    if isinstance(scene, Mesh):
        scene = scene.scene()
    elif isinstance(scene, SceneArrays):
        keep = scene
        scene = scene_from_arrays(keep)
    slots, ms = C.c_uint32(), (C.c_float * 3)()
    N.check(N.lib.sppm_tune_hash_slots(C.byref(cfg), C.byref(scene), C.byref(camera), device, passes,
                                       C.byref(slots), ms))
    return int(slots.value), [float(x) for x in ms]


def reduce_texture(d_texture: int, resolution: int, op: int, stream: int = 0) -> np.ndarray:
    """ReduceTexture on a device float4 texture (sppm_reduce_texture); returns the 1x1 texel."""
    out = (C.c_float * 4)()
    N.check(N.lib.sppm_reduce_texture(d_texture, resolution, op, out, stream))
    return np.array(list(out), dtype=np.float32)


class _PinnedBlock:
    def __init__(self, nbytes: int):
        self.ptr = C.c_void_p()
        N.check(N.lib.sppm_host_alloc(nbytes, C.byref(self.ptr)))

    def __del__(self):
        if getattr(self, "ptr", None) is not None and self.ptr.value:
            N.lib.sppm_host_free(self.ptr)
            self.ptr = None


def pinned_empty(shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked host memory (freed with the array)."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    block = _PinnedBlock(max(n, 1))
    buf = (C.c_char * max(n, 1)).from_address(block.ptr.value)
    buf._block = block  # the ctypes buffer keeps the allocation alive; numpy keeps the buffer
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)


def write_image(path, rgb: np.ndarray, fmt: str = "pfm") -> None:
    """Writes an [h, w, 3] image as read_image returns it (row 0 = bottom): 'pfm' and 'exr' keep the
    linear floats, 'ppm' writes 8-bit values (for display images)."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    h, w = rgb.shape[:2]
    N.check(N.lib.sppm_write_image_file(str(path).encode(), rgb.ctypes.data, w, h, {"pfm": 0, "ppm": 1, "exr": 2}[fmt]))


def debug_fpmath(fn: int, x: np.ndarray, y: np.ndarray | None = None) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    yy = None if y is None else np.ascontiguousarray(y, dtype=np.float32)
    out = np.empty_like(x)
    N.check(N.lib.sppm_debug_fpmath(fn, x.ctypes.data, None if yy is None else yy.ctypes.data, out.ctypes.data, x.size))
    return out
