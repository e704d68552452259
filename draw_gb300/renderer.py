"""Python mirror of the reference renderer's object model over the C ABI.

The reference (mororo18/draw, Rust) exposes ``Scene``, ``Camera``, ``Object``,
``Texture``, ``TextureMap`` and ``Canvas`` (src/renderer/scene/mod.rs,
scene/object.rs, canvas.rs). The classes here keep those names, argument
meanings and method names, and call the CUDA library ``libdrawgpu.so``
(include/draw_gpu.h) through ctypes. Where the reference panics (assert!,
unwrap, out-of-range slice), these raise ``DrawError`` carrying the library's
status code. There is no CPU fallback: importing this module on a machine
without the built library or without a GPU fails loudly.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libdrawgpu.so")

DG_OK = 0
STATUS = {
    1: "DG_E_INVALID", 2: "DG_E_INDEX", 3: "DG_E_TEXTURE_RANGE", 4: "DG_E_CAMERA", 5: "DG_E_DEPTH_UNINIT",
    6: "DG_E_CUDA", 7: "DG_E_OOM", 8: "DG_E_LIMIT", 9: "DG_E_TIMEOUT", 10: "DG_E_CANCELLED",
}

# Every symbol declared in include/draw_gpu.h, with its ctypes signature.
_P, _i32, _u32, _u64, _f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float
SIGNATURES = {
    "dg_ctx_create": (_i32, [_i32, _P]),
    "dg_ctx_destroy": (_i32, [_P]),
    "dg_status_string": (ctypes.c_char_p, [_i32]),
    "dg_ctx_synchronize": (_i32, [_P]),
    "dg_ctx_set_stream": (_i32, [_P, _P]),
    "dg_ctx_stream": (_P, [_P]),
    "dg_ctx_set_timing": (_i32, [_P, _i32]),
    "dg_ctx_kernel_times": (_i32, [_P, _P, _i32]),
    "dg_timeline_read": (_i32, [_P, _P, _i32]),
    "dg_ctx_last_stats": (_i32, [_P, _P, _i32]),
    "dg_check_division": (_i32, [_P, _i32, _u64, _u64, _P, _P, _P]),
    "dg_ctx_set_tuning": (_i32, [_P, _P]),
    "dg_ctx_get_tuning": (_i32, [_P, _P]),
    "dg_texmap_create": (_i32, [_P, _P, _u64, _u64, _u64, _u64, _P]),
    "dg_texmap_set_filter": (_i32, [_P, _i32, _i32]),
    "dg_scene_set_interpolation": (_i32, [_P, _i32, _i32]),
    "dg_object_create": (_i32, [_P, _P, _u64, _P, _u64, _P, _u64, _P, _u64, _P, _u64, _P]),
    "dg_object_destroy": (_i32, [_P, _i32]),
    "dg_scene_create": (_i32, [_P, _u64, _u64, _P]),
    "dg_scene_add_obj": (_i32, [_P, _i32, _i32, _P]),
    "dg_scene_set_camera": (_i32, [_P, _i32, _P, _P, _f32, _f32, _f32, _f32]),
    "dg_scene_camera_op": (_i32, [_P, _i32, _i32, _P]),
    "dg_scene_get_camera": (_i32, [_P, _i32, _P, _P]),
    "dg_scene_set_lights": (_i32, [_P, _i32, _P, _u32]),
    "dg_scene_set_exponent": (_i32, [_P, _i32, _i32]),
    "dg_scene_frame_setup": (_i32, [_P, _i32, _P, _P]),
    "dg_object_transparent_tris": (_i32, [_P, _i32, _u32, _P, _u64, _P]),
    "dg_canvas_create": (_i32, [_P, _u64, _u64, _P]),
    "dg_canvas_destroy": (_i32, [_P, _i32]),
    "dg_canvas_init_depth": (_i32, [_P, _i32, _f32]),
    "dg_canvas_apply_offset": (_i32, [_P, _i32, _i32, _i32]),
    "dg_canvas_resize": (_i32, [_P, _i32, _u64, _u64]),
    "dg_canvas_clear": (_i32, [_P, _i32]),
    "dg_canvas_read": (_i32, [_P, _i32, _P, _P]),
    "dg_canvas_read_async": (_i32, [_P, _i32, _P, _P]),
    "dg_canvas_read_wait": (_i32, [_P, _i32]),
    "dg_canvas_write": (_i32, [_P, _i32, _P, _P]),
    "dg_canvas_device_ptrs": (_i32, [_P, _i32, _P, _P]),
    "dg_canvas_size": (_i32, [_P, _i32, _P, _P]),
    "dg_canvas_draw_triangles_2d": (_i32, [_P, _i32, _P, _u32, _i32, _P]),
    "dg_canvas_read_rgba": (_i32, [_P, _i32, _P]),
    "dg_scene_render": (_i32, [_P, _i32, _i32]),
    "dg_render_batch": (_i32, [_P, _P, _P, _u32]),
    "dg_render_noalloc": (_i32, [_P, _P, _P, _u32, _P, _u32, _P, _P, _P, _P]),
    "dg_batch_create": (_i32, [_P, _P, _P, _u32, _P]),
    "dg_batch_render": (_i32, [_P]),
    "dg_batch_info": (_i32, [_P, _P, _i32]),
    "dg_batch_destroy": (_i32, [_P]),
    "dg_autotune": (_i32, [_P, _P, _P, _u32, _u32, _P, _P]),
    "dg_obj_parse": (_i32, [ctypes.c_char_p, _P]),
    "dg_obj_counts": (_i32, [_P, _P, _i32]),
    "dg_obj_arrays": (_i32, [_P, _P, _P, _P]),
    "dg_obj_mesh": (_i32, [_P, _u64, _P, _u64, _P, _P, _P, _u64]),
    "dg_obj_material": (_i32, [_P, _u64, _P, _P, _u64, _P, _P, _u64]),
    "dg_obj_name": (_i32, [_P, _P, _u64]),
    "dg_obj_free": (_i32, [_P]),
    "dg_server_create": (_i32, [_P, _u64, _u32, _u32, _P]),
    "dg_server_submit": (_i32, [_P, _P, _P]),
    "dg_server_wait": (_i32, [_P, _u64, _P, _P, _P]),
    "dg_server_stats": (_i32, [_P, _P, _i32]),
    "dg_server_reset_stats": (_i32, [_P]),
    "dg_server_cancel": (_i32, [_P, _u64]),
    "dg_server_inject_alloc_failure": (_i32, [_P, _u64]),
    "dg_server_destroy": (_i32, [_P]),
}


class DrawError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        super().__init__(f"{what}: {STATUS.get(status, status)}")
        self.status = status


class dg_material(ctypes.Structure):
    _fields_ = [("ka", ctypes.c_float * 3), ("kd", ctypes.c_float * 3), ("ks", ctypes.c_float * 3),
                ("alpha", ctypes.c_float), ("map_ka", ctypes.c_int32), ("map_kd", ctypes.c_int32)]


class dg_mesh_desc(ctypes.Structure):
    _fields_ = [("tris", ctypes.c_void_p), ("ntri", ctypes.c_uint64), ("texture_idx", ctypes.c_int32)]


MAX_LIGHTS = 8


class dg_request(ctypes.Structure):
    _fields_ = [("object", ctypes.c_int32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("cam_pos", ctypes.c_float * 3), ("cam_dir", ctypes.c_float * 3), ("near_", ctypes.c_float),
                ("far_", ctypes.c_float), ("fov_x_deg", ctypes.c_float), ("lights", (ctypes.c_float * 3) * MAX_LIGHTS),
                ("nlights", ctypes.c_uint32), ("exponent", ctypes.c_int32), ("clear_depth", ctypes.c_float),
                ("discard", ctypes.c_int32)]


# dg_render_noalloc's argument structs (include/draw_gpu.h).
NOALLOC_MAX_LIGHTS = 2


class dg_device_mesh(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_void_p), ("nrm", ctypes.c_void_p), ("uv", ctypes.c_void_p),
                ("tri_pos", ctypes.c_void_p), ("tri_uv", ctypes.c_void_p), ("tri_nrm", ctypes.c_void_p),
                ("nv", ctypes.c_uint32), ("nn", ctypes.c_uint32), ("nuv", ctypes.c_uint32), ("ntri", ctypes.c_uint32)]


class dg_device_texmap(ctypes.Structure):
    _fields_ = [("bytes", ctypes.c_void_p), ("len", ctypes.c_uint64), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("components", ctypes.c_uint32)]


class dg_frame_params(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("canvas_width", ctypes.c_uint32),
                ("canvas_height", ctypes.c_uint32), ("cam_pos", ctypes.c_float * 3), ("cam_dir", ctypes.c_float * 3),
                ("near_", ctypes.c_float), ("far_", ctypes.c_float), ("fov_x_deg", ctypes.c_float),
                ("lights", (ctypes.c_float * 3) * NOALLOC_MAX_LIGHTS), ("nlights", ctypes.c_uint32),
                ("exponent", ctypes.c_int32), ("clear_depth", ctypes.c_float), ("offset_x", ctypes.c_int32),
                ("offset_y", ctypes.c_int32)]


_lib = None


def load_library() -> ctypes.CDLL:
    """Loads the in-tree libdrawgpu.so (or the in-tree library that
    DRAW_GB300_LIB names, e.g. the DRAW_CHECKED build); raises if it has not
    been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("DRAW_GB300_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with draw_gb300._build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


# Extension modes (dg_scene_set_interpolation, dg_texmap_set_filter); the
# defaults are the reference's behaviour.
INTERP_AFFINE, INTERP_PERSPECTIVE = 0, 1
FILTER_NEAREST, FILTER_BILINEAR = 0, 1

# Kernels of one render job in launch order (dg_ctx_kernel_times).
KERNELS = ["vertex", "cull", "setup_raster", "queue_raster", "resolve"]
# dg_tuning fields in order.
TUNING_KEYS = ["small_max_px", "setup_blocks_per_sm", "queue_blocks_per_sm", "cull_blocks_per_sm", "record_limit",
               "tile_rows", "item_units"]
# dg_ctx_last_stats entries in order.
STATS_KEYS = ["vertices", "triangles", "queued_triangles", "queued_units", "covered_pixels", "inplace_triangles",
              "h2d_bytes", "launches", "survivors", "triangle_records", "clip_rows", "small_triangles", "tile_rows",
              "small_max_px"]


def _chk(st: int, what: str):
    if st != DG_OK:
        raise DrawError(st, what)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """One CUDA device and stream; owns every resource created through it."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        _chk(self.lib.dg_ctx_create(device, ctypes.byref(h)), "dg_ctx_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.dg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        _chk(self.lib.dg_ctx_synchronize(self.h), "synchronize")

    def set_stream(self, stream_ptr: int | None):
        _chk(self.lib.dg_ctx_set_stream(self.h, stream_ptr), "set_stream")

    def set_timing(self, on: bool):
        _chk(self.lib.dg_ctx_set_timing(self.h, 1 if on else 0), "set_timing")

    def kernel_times(self) -> dict:
        ms = (ctypes.c_float * len(KERNELS))()
        _chk(self.lib.dg_ctx_kernel_times(self.h, ms, len(KERNELS)), "kernel_times")
        return dict(zip(KERNELS, list(ms)))

    def timeline(self) -> dict:
        """dg_timeline_read (DRAW_TIMELINE builds): per kernel, microseconds after the
        first k_vertex block's start: (first block start, first wait passed, last
        wait passed, last block end), None where nothing was recorded."""
        raw = (ctypes.c_uint64 * (4 * len(KERNELS)))()
        _chk(self.lib.dg_timeline_read(self.h, raw, len(raw)), "timeline")
        t0 = raw[0]
        return {k: tuple(None if raw[4 * i + j] == 0 or t0 == 0 else (raw[4 * i + j] - t0) / 1000.0
                         for j in range(4)) for i, k in enumerate(KERNELS)}

    def set_tuning(self, **knobs):
        """Raster knobs (TUNING_KEYS): in-warp raster threshold (bounding-box pixels) and grid
        sizes per SM; keys left out keep their value. Results do not depend on them, only speed."""
        t = self.get_tuning()
        for k, v in knobs.items():
            if k not in t:
                raise KeyError(k)
            if v is not None:
                t[k] = int(v)
        raw = (ctypes.c_uint32 * len(TUNING_KEYS))(*[t[k] for k in TUNING_KEYS])
        _chk(self.lib.dg_ctx_set_tuning(self.h, raw), "set_tuning")

    def get_tuning(self) -> dict:
        raw = (ctypes.c_uint32 * len(TUNING_KEYS))()
        _chk(self.lib.dg_ctx_get_tuning(self.h, raw), "get_tuning")
        return dict(zip(TUNING_KEYS, list(raw)))

    def last_stats(self) -> dict:
        v = (ctypes.c_uint64 * len(STATS_KEYS))()
        _chk(self.lib.dg_ctx_last_stats(self.h, v, len(STATS_KEYS)), "last_stats")
        return dict(zip(STATS_KEYS, list(v)))

    def check_division(self, mode: int, samples: int, seed: int = 1) -> tuple:
        """dg_check_division: (mismatches, first mismatching a, b) of one sample family."""
        n, a, b = ctypes.c_uint64(), ctypes.c_float(), ctypes.c_float()
        _chk(self.lib.dg_check_division(self.h, mode, samples, seed, ctypes.byref(n), ctypes.byref(a),
                                        ctypes.byref(b)), "check_division")
        return n.value, a.value, b.value

    def render_batch(self, scenes: list, canvases: list):
        """The batched form: all frames in one launch per pipeline stage."""
        s = np.array([x.id for x in scenes], np.int32)
        c = np.array([x.id for x in canvases], np.int32)
        _chk(self.lib.dg_render_batch(self.h, _ptr(s), _ptr(c), len(scenes)), "render_batch")

    def batch(self, scenes: list, canvases: list) -> "Batch":
        """The batched form replayed from a CUDA graph (dg_batch_*)."""
        return Batch(self, scenes, canvases)

    def autotune(self, scenes: list, canvases: list, reps: int = 3) -> tuple[dict, float]:
        """dg_autotune over these frames: sets and returns the fastest tuning and its ms per render."""
        s = np.array([x.id for x in scenes], np.int32)
        c = np.array([x.id for x in canvases], np.int32)
        raw = (ctypes.c_uint32 * len(TUNING_KEYS))()
        ms = ctypes.c_float()
        _chk(self.lib.dg_autotune(self.h, _ptr(s), _ptr(c), len(scenes), int(reps), raw, ctypes.byref(ms)),
             "autotune")
        return dict(zip(TUNING_KEYS, list(raw))), float(ms.value)


BATCH_INFO_KEYS = ["frames", "captures", "replays", "kernels_per_replay", "h2d_bytes_per_replay"]


class Batch:
    """n (scene, canvas) frames rendered as one job whose launch sequence is a
    CUDA graph captured once and replayed by each render() (dg_batch_render).
    Cameras and lights may change between renders; shape changes re-capture."""

    def __init__(self, ctx: Context, scenes: list, canvases: list):
        self.ctx = ctx
        s = np.array([x.id for x in scenes], np.int32)
        c = np.array([x.id for x in canvases], np.int32)
        h = ctypes.c_void_p()
        _chk(ctx.lib.dg_batch_create(ctx.h, _ptr(s), _ptr(c), len(scenes), ctypes.byref(h)), "batch_create")
        self.h = h

    def render(self):
        _chk(self.ctx.lib.dg_batch_render(self.h), "batch_render")

    def info(self) -> dict:
        v = (ctypes.c_uint64 * len(BATCH_INFO_KEYS))()
        _chk(self.ctx.lib.dg_batch_info(self.h, v, len(BATCH_INFO_KEYS)), "batch_info")
        return dict(zip(BATCH_INFO_KEYS, list(v)))

    def close(self):
        if self.h:
            self.ctx.lib.dg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class TextureMap:
    """TextureMap::new(img, width, height, components), scene/mod.rs:113-126."""

    def __init__(self, img, width: int, height: int, components: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        a = np.ascontiguousarray(img, dtype=np.uint8).reshape(-1)
        out = ctypes.c_int32()
        _chk(self.ctx.lib.dg_texmap_create(self.ctx.h, _ptr(a), a.size, width, height, components,
                                           ctypes.byref(out)), "TextureMap::new")
        self.id = out.value
        self.width, self.height, self.components = width, height, components

    def set_filter(self, filt: int):
        """Extension (no counterpart in the reference): FILTER_NEAREST (the
        reference's get_rgb_slice) or FILTER_BILINEAR (dg_texmap_set_filter)."""
        _chk(self.ctx.lib.dg_texmap_set_filter(self.ctx.h, self.id, int(filt)), "TextureMap::set_filter")

    @staticmethod
    def load_from_file(path: str, ctx: Context | None = None) -> "TextureMap":
        """TextureMap::load_from_file (scene/mod.rs:174-202): 3- or 4-component images only."""
        from . import imageio

        img, w, h, comps = imageio.read_image(path)
        if comps not in (3, 4):
            raise DrawError(1, f"TextureMap::load_from_file {path}: {comps} components")
        return TextureMap(img, w, h, comps, ctx)


@dataclass
class Texture:
    """The reference's material (scene/mod.rs:206-216); map_* = TextureMap or None
    for the 1x1 white default map."""

    name: str = "default"
    ka: tuple = (0.9, 0.9, 0.9)
    kd: tuple = (0.4, 0.4, 0.4)
    ks: tuple = (0.5, 0.5, 0.5)
    alpha: float = 1.0
    map_ka: TextureMap | None = None
    map_kd: TextureMap | None = None

    @staticmethod
    def default() -> "Texture":  # scene/mod.rs:237-252
        return Texture()

    @staticmethod
    def with_diffuse_map(diff_map: TextureMap) -> "Texture":  # scene/mod.rs:219-234
        return Texture("default", (1.0, 1.0, 1.0), (1.0, 1.0, 1.0), (1.0, 1.0, 1.0), 1.0, None, diff_map)


@dataclass
class IndexedMesh:
    """scene/mesh.rs:30-35: triangles as (T, 9) indices (position[3], texture[3], normal[3])."""

    name: str
    triangles: np.ndarray
    texture_idx: int = 0


@dataclass
class MeshInfo:
    name: str
    triangle_count: int
    texture_name: str | None


@dataclass
class ObjectInfo:
    id: int
    name: str
    mesh_info_list: list = field(default_factory=list)


class Object:
    """Object::new(name, vertices, normals, texture_vertices, meshes, textures), object.rs:34-71."""

    def __init__(self, name: str, vertices, normals, texture_vertices, meshes: list, textures: list,
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.name = name
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        uv = np.asarray(texture_vertices if texture_vertices is not None else np.zeros((0, 3)), np.float32)
        if uv.ndim == 2 and uv.shape[1] == 2:
            uv = np.concatenate([uv, np.zeros((uv.shape[0], 1), np.float32)], 1)
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 3)
        tris = [np.ascontiguousarray(m.triangles, np.uint32).reshape(-1, 9) for m in meshes]
        md = (dg_mesh_desc * max(1, len(meshes)))()
        for i, (m, t) in enumerate(zip(meshes, tris)):
            md[i].tris = t.ctypes.data_as(ctypes.c_void_p)
            md[i].ntri = t.shape[0]
            md[i].texture_idx = m.texture_idx
        mats = (dg_material * max(1, len(textures)))()
        for i, t in enumerate(textures):
            mats[i].ka[:] = list(t.ka)
            mats[i].kd[:] = list(t.kd)
            mats[i].ks[:] = list(t.ks)
            mats[i].alpha = t.alpha
            mats[i].map_ka = t.map_ka.id if t.map_ka is not None else -1
            mats[i].map_kd = t.map_kd.id if t.map_kd is not None else -1
        out = ctypes.c_int32()
        _chk(self.ctx.lib.dg_object_create(self.ctx.h, _ptr(v), v.shape[0], _ptr(n), n.shape[0], _ptr(uv),
                                           uv.shape[0], ctypes.cast(md, ctypes.c_void_p), len(meshes),
                                           ctypes.cast(mats, ctypes.c_void_p), len(textures), ctypes.byref(out)),
             "Object::new")
        self.id = out.value
        self.meshes = meshes
        self.textures = textures

    @staticmethod
    def load_from_file(filename: str, ctx: Context | None = None) -> "Object":
        """Object::load_from_file (object.rs:106-454): the OBJ file and its MTL
        libraries parsed by the library (dg_obj_*), texture maps decoded here."""
        ctx = ctx or default_context()
        lib = ctx.lib
        h = ctypes.c_void_p()
        _chk(lib.dg_obj_parse(os.fsencode(filename), ctypes.byref(h)), f"Object::load_from_file {filename}")
        try:
            cnt = (ctypes.c_uint64 * 6)()
            _chk(lib.dg_obj_counts(h, cnt, 6), "obj counts")
            nv, nn, nuv, nmesh, nmat = (int(x) for x in cnt[:5])
            v = np.zeros((nv, 3), np.float32)
            n = np.zeros((nn, 3), np.float32)
            uv = np.zeros((nuv, 3), np.float32)
            _chk(lib.dg_obj_arrays(h, _ptr(v), _ptr(n), _ptr(uv)), "obj arrays")
            name = ctypes.create_string_buffer(1024)
            meshes = []
            for i in range(nmesh):
                nt, ti = ctypes.c_uint64(), ctypes.c_int32()
                _chk(lib.dg_obj_mesh(h, i, None, 0, ctypes.byref(nt), ctypes.byref(ti), name, 1024), "obj mesh")
                t = np.zeros((nt.value, 9), np.uint32)
                _chk(lib.dg_obj_mesh(h, i, _ptr(t), t.size, ctypes.byref(nt), ctypes.byref(ti), name, 1024),
                     "obj mesh")
                meshes.append(IndexedMesh(name.value.decode(), t, ti.value))
            maps: dict = {}
            textures = []
            pa, pd = ctypes.create_string_buffer(4096), ctypes.create_string_buffer(4096)
            for i in range(nmat):
                m = dg_material()
                _chk(lib.dg_obj_material(h, i, ctypes.byref(m), name, 1024, pa, pd, 4096), "obj material")
                tm = []
                for p in (pa.value.decode(), pd.value.decode()):
                    if p and p not in maps:
                        maps[p] = TextureMap.load_from_file(p, ctx)
                    tm.append(maps[p] if p else None)
                textures.append(Texture(name.value.decode(), tuple(m.ka), tuple(m.kd), tuple(m.ks), m.alpha, tm[0],
                                        tm[1]))
            _chk(lib.dg_obj_name(h, name, 1024), "obj name")
            return Object(name.value.decode(), v, n, uv, meshes, textures, ctx)
        finally:
            lib.dg_obj_free(h)

    @staticmethod
    def load_from_directory(directory: str, ctx: Context | None = None) -> list:
        """Object::load_from_directory (object.rs:73-103): every .obj file of the directory."""
        if not os.path.isdir(directory):
            return []
        return [Object.load_from_file(os.path.join(directory, f), ctx) for f in sorted(os.listdir(directory))
                if f.endswith(".obj") and os.path.isfile(os.path.join(directory, f))]

    def transparent_triangles(self, mesh: int) -> np.ndarray:
        """The current (painter's sort) order of transparent mesh `mesh` as (T, 9)
        indices; Scene::render re-sorts it every frame and keeps it (scene/mod.rs:1100-1115)."""
        n = ctypes.c_uint64()
        _chk(self.ctx.lib.dg_object_transparent_tris(self.ctx.h, self.id, mesh, None, 0, ctypes.byref(n)),
             "transparent_tris")
        out = np.zeros((n.value, 9), np.uint32)
        if n.value:
            _chk(self.ctx.lib.dg_object_transparent_tris(self.ctx.h, self.id, mesh, _ptr(out), out.size,
                                                         ctypes.byref(n)), "transparent_tris")
        return out

    def mesh_info_list(self) -> list:  # object.rs:456-476 (opaque meshes first, then transparent)
        transparent = [self.textures[m.texture_idx].alpha < 1.0 for m in self.meshes]
        order = [m for m, t in zip(self.meshes, transparent) if not t] + \
                [m for m, t in zip(self.meshes, transparent) if t]
        return [MeshInfo(m.name, int(np.asarray(m.triangles).reshape(-1, 9).shape[0]),
                         self.textures[m.texture_idx].name) for m in order]


class Camera:
    """Scene.camera (scene/mod.rs:282-594): movement methods act on the scene's camera."""

    def __init__(self, scene: "Scene"):
        self._s = scene

    def _op(self, op: int, *args):
        a = np.zeros(3, np.float32)
        a[: len(args)] = args
        _chk(self._s.ctx.lib.dg_scene_camera_op(self._s.ctx.h, self._s.id, op, _ptr(a)), "camera")

    def move_up(self, d): self._op(0, d)
    def move_down(self, d): self._op(1, d)
    def move_left(self, d): self._op(2, d)
    def move_right(self, d): self._op(3, d)
    def move_foward(self, d): self._op(4, d)  # noqa: E704 (reference spelling)
    def move_backward(self, d): self._op(5, d)
    def rotate_origin(self, theta_deg): self._op(6, theta_deg)
    def set_pos(self, pos): self._op(7, *pos)

    def get_pos(self) -> np.ndarray:
        return self._get()[0]

    def get_direction(self) -> np.ndarray:
        return self._get()[1]

    def _get(self):
        p = np.zeros(3, np.float32)
        d = np.zeros(3, np.float32)
        _chk(self._s.ctx.lib.dg_scene_get_camera(self._s.ctx.h, self._s.id, _ptr(p), _ptr(d)), "camera")
        return p, d

    def reset(self, pos, direction, ratio, near=-10.0, far=-510.0, fov_x=135.0):
        """Camera::new(pos, dir, ratio) with explicit projection constants."""
        p = np.asarray(pos, np.float32)
        d = np.asarray(direction, np.float32)
        _chk(self._s.ctx.lib.dg_scene_set_camera(self._s.ctx.h, self._s.id, _ptr(p), _ptr(d), ratio, near, far,
                                                 fov_x), "Camera::new")


class Scene:
    """Scene::new(width, height) (scene/mod.rs:760-786) and Scene::render."""

    def __init__(self, width: int, height: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        out = ctypes.c_int32()
        _chk(self.ctx.lib.dg_scene_create(self.ctx.h, width, height, ctypes.byref(out)), "Scene::new")
        self.id = out.value
        self.width, self.height = width, height
        self.camera = Camera(self)
        self._next_object_id = 0

    def add_obj(self, obj: Object) -> ObjectInfo:
        oid = ctypes.c_uint32()
        _chk(self.ctx.lib.dg_scene_add_obj(self.ctx.h, self.id, obj.id, ctypes.byref(oid)), "Scene::add_obj")
        return ObjectInfo(oid.value, obj.name, obj.mesh_info_list())

    def move_camera_direction(self, dx: int, dy: int):
        self.camera._op(8, dx, dy)

    def set_lights(self, lights):
        l = np.ascontiguousarray(lights, np.float32).reshape(-1, 3)
        _chk(self.ctx.lib.dg_scene_set_lights(self.ctx.h, self.id, _ptr(l), l.shape[0]), "set_lights")

    def set_exponent(self, e: int):
        _chk(self.ctx.lib.dg_scene_set_exponent(self.ctx.h, self.id, int(e)), "set_exponent")

    def set_interpolation(self, mode: int):
        """Extension (no counterpart in the reference): INTERP_AFFINE (the
        reference's screen-space interpolation) or INTERP_PERSPECTIVE
        (dg_scene_set_interpolation)."""
        _chk(self.ctx.lib.dg_scene_set_interpolation(self.ctx.h, self.id, int(mode)), "set_interpolation")

    def frame_setup(self):
        M = np.zeros(16, np.float32)
        P = np.zeros(24, np.float32)
        _chk(self.ctx.lib.dg_scene_frame_setup(self.ctx.h, self.id, _ptr(M), _ptr(P)), "frame_setup")
        return M.reshape(4, 4), P.reshape(6, 4)

    def render(self, canvas: "Canvas"):
        _chk(self.ctx.lib.dg_scene_render(self.ctx.h, self.id, canvas.id), "Scene::render")


class Canvas:
    """Canvas (canvas.rs:353-983): BGRA colour buffer (row 0 = top) and f32 depth."""

    def __init__(self, width: int, height: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        out = ctypes.c_int32()
        _chk(self.ctx.lib.dg_canvas_create(self.ctx.h, width, height, ctypes.byref(out)), "Canvas::new")
        self.id = out.value
        self.width, self.height = width, height

    def init_depth(self, depth: float):
        _chk(self.ctx.lib.dg_canvas_init_depth(self.ctx.h, self.id, depth), "init_depth")

    def apply_offset(self, x: int, y: int):
        _chk(self.ctx.lib.dg_canvas_apply_offset(self.ctx.h, self.id, x, y), "apply_offset")

    def resize(self, width: int, height: int):
        _chk(self.ctx.lib.dg_canvas_resize(self.ctx.h, self.id, width, height), "resize")
        self.width, self.height = width, height

    def clear(self):
        _chk(self.ctx.lib.dg_canvas_clear(self.ctx.h, self.id), "clear")

    @staticmethod
    def pixel_bytes() -> int:
        return 4

    def size_bytes(self) -> int:
        return 4 * self.width * self.height

    def as_bytes_slice(self) -> bytes:
        return self.read()[0].tobytes()

    def read(self, depth: bool = True):
        """(bgra (H, W, 4) uint8 with row 0 = top, depth (H, W) float32 with row 0 = y 0)."""
        bgra = np.empty((self.height, self.width, 4), np.uint8)
        d = np.empty((self.height, self.width), np.float32) if depth else None
        _chk(self.ctx.lib.dg_canvas_read(self.ctx.h, self.id, _ptr(bgra), _ptr(d)), "Canvas::read")
        return bgra, d

    def read_rgba(self) -> np.ndarray:
        """(H, W, 4) RGBA bytes, row 0 = top: the frame Application::export_frame_as writes."""
        out = np.empty((self.height, self.width, 4), np.uint8)
        _chk(self.ctx.lib.dg_canvas_read_rgba(self.ctx.h, self.id, _ptr(out)), "read_rgba")
        return out

    def export_frame_as(self, path: str):
        """Application::export_frame_as (app/mod.rs:316-379): PNG with 4 components
        (the padding byte as alpha), or binary PPM (RGB); JPEG is not encoded here."""
        from . import imageio

        if path.lower().endswith(".png"):
            imageio.write_png(path, self.read_rgba())
        elif path.lower().endswith(".ppm"):
            imageio.write_ppm(path, self.read_rgba())
        else:
            raise DrawError(1, f"export_frame_as {path}: PNG and PPM are written")

    def draw_triangles(self, verts, texture_map: "TextureMap | None" = None, clips=None):
        """Canvas::draw_triangle (canvas.rs:435-575) for n triangles in order: verts
        (n, 3, 8) = (x, y, u, v, r, g, b, alpha) per vertex; clips (n, 4) or None."""
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 24)
        c = None if clips is None else np.ascontiguousarray(clips, np.uint64).reshape(-1, 4)
        tid = texture_map.id if texture_map is not None else -1
        _chk(self.ctx.lib.dg_canvas_draw_triangles_2d(self.ctx.h, self.id, _ptr(v), v.shape[0], tid, _ptr(c)),
             "Canvas::draw_triangle")

    def read_into(self, bgra: np.ndarray, depth: np.ndarray | None):
        _chk(self.ctx.lib.dg_canvas_read(self.ctx.h, self.id, _ptr(bgra), _ptr(depth)), "Canvas::read")

    def read_async(self, bgra: np.ndarray | None, depth: np.ndarray | None = None):
        """dg_canvas_read_async: starts the copy into the (pinned) host arrays and
        returns; the arrays are valid after read_wait()."""
        _chk(self.ctx.lib.dg_canvas_read_async(self.ctx.h, self.id, _ptr(bgra), _ptr(depth)), "Canvas::read_async")

    def read_wait(self):
        _chk(self.ctx.lib.dg_canvas_read_wait(self.ctx.h, self.id), "Canvas::read_wait")

    def write(self, bgra: np.ndarray | None, depth: np.ndarray | None):
        b = None if bgra is None else np.ascontiguousarray(bgra, np.uint8)
        d = None if depth is None else np.ascontiguousarray(depth, np.float32)
        _chk(self.ctx.lib.dg_canvas_write(self.ctx.h, self.id, _ptr(b), _ptr(d)), "Canvas::write")


# ------------------------------------------------------------ scene builder
@dataclass
class BuiltScene:
    scene: Scene
    canvas: Canvas
    objects: list
    texmaps: list


def build_scene(desc, ctx: Context | None = None) -> BuiltScene:
    """Uploads a draw_gb300.scenes.SceneDesc: texture maps, objects, scene, camera, canvas."""
    ctx = ctx or default_context()
    texmaps = [TextureMap(t.img, t.width, t.height, t.comps, ctx) for t in desc.textures]
    for t, m in zip(desc.textures, texmaps):
        if getattr(t, "filter", 0):
            m.set_filter(t.filter)
    scene = Scene(desc.width, desc.height, ctx)
    scene.camera.reset(desc.cam_pos, desc.cam_dir, float(desc.ratio), desc.near, desc.far, desc.fov_x)
    scene.set_lights(desc.lights)
    scene.set_exponent(desc.exponent)
    if getattr(desc, "interpolation", 0):
        scene.set_interpolation(desc.interpolation)
    objects = []
    for o in desc.objects:
        mats = [Texture(f"m{i}", m.ka, m.kd, m.ks, m.alpha, texmaps[m.map_ka] if m.map_ka >= 0 else None,
                        texmaps[m.map_kd] if m.map_kd >= 0 else None) for i, m in enumerate(o.materials)]
        meshes = [IndexedMesh(f"mesh{i}", m.tris, m.texture_idx) for i, m in enumerate(o.meshes)]
        ob = Object("object", o.vertices, o.normals, o.uvs, meshes, mats, ctx)
        scene.add_obj(ob)
        objects.append(ob)
    cw, ch = desc.canvas_size
    canvas = Canvas(cw, ch, ctx)
    canvas.init_depth(desc.clear_depth)
    canvas.apply_offset(*desc.offset)
    return BuiltScene(scene, canvas, objects, texmaps)


def upload_object(o, texmaps: list, ctx: Context) -> Object:
    """Uploads one scenes.ObjectDesc whose material maps index `texmaps`."""
    mats = [Texture(f"m{i}", m.ka, m.kd, m.ks, m.alpha, texmaps[m.map_ka] if m.map_ka >= 0 else None,
                    texmaps[m.map_kd] if m.map_kd >= 0 else None) for i, m in enumerate(o.materials)]
    meshes = [IndexedMesh(f"mesh{i}", m.tris, m.texture_idx) for i, m in enumerate(o.meshes)]
    return Object("object", o.vertices, o.normals, o.uvs, meshes, mats, ctx)


class Server:
    """The continuous-batching render server (dg_server_*): submit requests from
    any thread, wait for each one, read latency percentiles."""

    def __init__(self, ctx: Context, budget_bytes: int, max_batch: int = 64, streams: int = 3):
        self.ctx = ctx
        h = ctypes.c_void_p()
        _chk(ctx.lib.dg_server_create(ctx.h, int(budget_bytes), max_batch, streams, ctypes.byref(h)), "server")
        self.h = h

    @staticmethod
    def request(obj: Object, width, height, cam_pos, cam_dir, near, far, fov_x, lights, exponent=2,
                clear_depth=float("inf"), discard=False) -> dg_request:
        r = dg_request()
        r.object, r.width, r.height = obj.id, width, height
        r.cam_pos[:] = [float(x) for x in cam_pos]
        r.cam_dir[:] = [float(x) for x in cam_dir]
        r.near_, r.far_, r.fov_x_deg = near, far, fov_x
        lights = np.asarray(lights, np.float32).reshape(-1, 3)
        for i, l in enumerate(lights):
            r.lights[i][:] = [float(x) for x in l]
        r.nlights, r.exponent, r.clear_depth, r.discard = len(lights), exponent, clear_depth, 1 if discard else 0
        return r

    def submit(self, req: dg_request) -> int:
        t = ctypes.c_uint64()
        _chk(self.ctx.lib.dg_server_submit(self.h, ctypes.byref(req), ctypes.byref(t)), "server submit")
        return t.value

    def wait(self, ticket: int, width: int = 0, height: int = 0, read: bool = False):
        """Returns (bgra, depth, latency_ms); the frame only when read=True."""
        lat = ctypes.c_double()
        bgra = np.empty((height, width, 4), np.uint8) if read else None
        depth = np.empty((height, width), np.float32) if read else None
        _chk(self.ctx.lib.dg_server_wait(self.h, ticket, _ptr(bgra), _ptr(depth), ctypes.byref(lat)), "server wait")
        return bgra, depth, lat.value

    def stats(self) -> dict:
        v = (ctypes.c_double * 9)()
        _chk(self.ctx.lib.dg_server_stats(self.h, v, 9), "server stats")
        keys = ["completed", "p50_ms", "p99_ms", "max_ms", "batches", "mean_batch", "peak_bytes", "error",
                "allocations"]
        return dict(zip(keys, list(v)))

    def cancel(self, ticket: int):
        """dg_server_cancel: a request not admitted yet completes with DG_E_CANCELLED."""
        _chk(self.ctx.lib.dg_server_cancel(self.h, ticket), "server cancel")

    def inject_alloc_failure(self, ticket: int):
        """dg_server_inject_alloc_failure (test hook): the request's buffer allocation fails."""
        _chk(self.ctx.lib.dg_server_inject_alloc_failure(self.h, ticket), "server inject")

    def reset_stats(self):
        _chk(self.ctx.lib.dg_server_reset_stats(self.h), "server reset_stats")

    def close(self):
        if self.h:
            self.ctx.lib.dg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
