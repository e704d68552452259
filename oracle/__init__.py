"""CPU oracle for the draw rasterization path (TEST INFRASTRUCTURE).

This package is the parity checker, not the product. Only ``tests/``, the smoke
check in ``__graft_entry__.py`` and the CPU-baseline leg of ``bench.py`` may load
it. It wraps ``draw_oracle.cpp``, a C++ restatement of the reference renderer
(mororo18/draw, ``src/renderer/{linalg.rs,canvas.rs,scene/mod.rs}``), built by
``oracle/build.py`` into ``oracle/liboracle.so``.

Parity is unpinned by the reference itself: the reference has no tests and no
golden data, and it cannot be built here (Rust, no toolchain).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")

OR_OK = 0


class OracleError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what}: oracle error {code}")
        self.code = code


class or_material(ctypes.Structure):
    _fields_ = [
        ("ka", ctypes.c_float * 3),
        ("kd", ctypes.c_float * 3),
        ("ks", ctypes.c_float * 3),
        ("alpha", ctypes.c_float),
        ("map_ka", ctypes.c_int32),
        ("map_kd", ctypes.c_int32),
    ]


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _b

        _b.build()
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    i32, u32, u64, f32 = ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float
    sig = {
        "or_ctx_new": (P, []),
        "or_ctx_free": (None, [P]),
        "or_texmap_new": (i32, [P, P, u64, u64, u64, u64]),
        "or_object_new": (i32, [P, P, u64, P, u64, P, u64, P, P, P, u64, P, u64]),
        "or_scene_new": (i32, [P, u64, u64]),
        "or_scene_add_obj": (i32, [P, i32, i32]),
        "or_scene_set_camera": (i32, [P, i32, P, P, f32, f32, f32, f32]),
        "or_scene_set_lights": (i32, [P, i32, P, u32]),
        "or_scene_set_exponent": (i32, [P, i32, i32]),
        "or_scene_set_interpolation": (i32, [P, i32, i32]),
        "or_texmap_set_filter": (i32, [P, i32, i32]),
        "or_scene_camera_op": (i32, [P, i32, i32, P]),
        "or_scene_get_camera": (i32, [P, i32, P, P]),
        "or_scene_frame_setup": (i32, [P, i32, P, P]),
        "or_canvas_new": (i32, [P, u64, u64]),
        "or_canvas_init_depth": (i32, [P, i32, f32]),
        "or_canvas_apply_offset": (i32, [P, i32, i32, i32]),
        "or_canvas_resize": (i32, [P, i32, u64, u64]),
        "or_canvas_clear": (i32, [P, i32]),
        "or_canvas_read": (i32, [P, i32, P, P]),
        "or_canvas_write": (i32, [P, i32, P, P]),
        "or_scene_render": (i32, [P, i32, i32]),
        "or_object_transparent_tris": (i32, [P, i32, u32, P, u64]),
        "or_canvas_draw_triangle_2d": (i32, [P, i32, P, i32, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def _chk(rc: int, what: str) -> int:
    if rc < 0:
        raise OracleError(-rc, what)
    return rc


@dataclass
class OracleFrame:
    bgra: np.ndarray  # (H, W, 4) uint8, row 0 = top of the screen (reference memory order)
    depth: np.ndarray  # (H, W) float32, row 0 = screen y 0 (bottom), reference indexing y*W+x


class Oracle:
    """Stateful CPU renderer with the reference's object model (Scene, Object, Canvas)."""

    def __init__(self):
        self.lib = load()
        self.ctx = self.lib.or_ctx_new()
        self._keep = []

    def close(self):
        if self.ctx:
            self.lib.or_ctx_free(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- resources ---------------------------------------------------------
    def texmap(self, img: np.ndarray, width: int, height: int, comps: int) -> int:
        img = np.ascontiguousarray(img, dtype=np.uint8).reshape(-1)
        return _chk(self.lib.or_texmap_new(self.ctx, _ptr(img), img.size, width, height, comps), "texmap")

    def object(self, vertices, normals, uvs, meshes, materials) -> int:
        """meshes: list of (tris (T,9) uint32, texture_idx); materials: list of dicts
        with ka, kd, ks, alpha, map_ka, map_kd (texmap handles or -1)."""
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        uv = np.asarray(uvs, dtype=np.float32)
        if uv.ndim == 2 and uv.shape[1] == 2:
            uv = np.concatenate([uv, np.zeros((uv.shape[0], 1), np.float32)], axis=1)
        uv = np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 3)
        tris = np.ascontiguousarray(
            np.concatenate([np.asarray(m[0], dtype=np.uint32).reshape(-1, 9) for m in meshes])
            if meshes
            else np.zeros((0, 9), np.uint32),
            dtype=np.uint32,
        )
        ntri = np.array([np.asarray(m[0]).reshape(-1, 9).shape[0] for m in meshes], dtype=np.uint64)
        mtex = np.array([m[1] for m in meshes], dtype=np.int32)
        mats = (or_material * max(1, len(materials)))()
        for i, m in enumerate(materials):
            mats[i].ka[:] = list(m["ka"])
            mats[i].kd[:] = list(m["kd"])
            mats[i].ks[:] = list(m["ks"])
            mats[i].alpha = m["alpha"]
            mats[i].map_ka = m["map_ka"]
            mats[i].map_kd = m["map_kd"]
        rc = self.lib.or_object_new(
            self.ctx, _ptr(v), v.shape[0], _ptr(n), n.shape[0], _ptr(uv), uv.shape[0], _ptr(tris),
            _ptr(ntri), _ptr(mtex), len(meshes), ctypes.cast(mats, ctypes.c_void_p), len(materials),
        )
        return _chk(rc, "object")

    def scene(self, width: int, height: int) -> int:
        return _chk(self.lib.or_scene_new(self.ctx, width, height), "scene")

    def add_obj(self, scene: int, obj: int) -> int:
        return _chk(self.lib.or_scene_add_obj(self.ctx, scene, obj), "add_obj")

    def set_camera(self, scene, pos, direction, ratio, near=-10.0, far=-510.0, fov_x=135.0):
        p = np.asarray(pos, np.float32)
        d = np.asarray(direction, np.float32)
        _chk(self.lib.or_scene_set_camera(self.ctx, scene, _ptr(p), _ptr(d), ratio, near, far, fov_x), "camera")

    def set_lights(self, scene, lights):
        l = np.ascontiguousarray(lights, dtype=np.float32).reshape(-1, 3)
        _chk(self.lib.or_scene_set_lights(self.ctx, scene, _ptr(l), l.shape[0]), "lights")

    def set_exponent(self, scene, e: int):
        _chk(self.lib.or_scene_set_exponent(self.ctx, scene, e), "exponent")

    def set_interpolation(self, scene, mode: int):
        """Extension: 0 = the reference's screen-space interpolation, 1 = perspective-correct."""
        _chk(self.lib.or_scene_set_interpolation(self.ctx, scene, mode), "interpolation")

    def set_filter(self, texmap: int, filt: int):
        """Extension: 0 = the reference's nearest texel, 1 = bilinear."""
        _chk(self.lib.or_texmap_set_filter(self.ctx, texmap, filt), "filter")

    def camera_op(self, scene, op: int, v):
        a = np.zeros(3, np.float32)
        a[: len(v)] = v
        _chk(self.lib.or_scene_camera_op(self.ctx, scene, op, _ptr(a)), "camera_op")

    def get_camera(self, scene):
        p = np.zeros(3, np.float32)
        d = np.zeros(3, np.float32)
        _chk(self.lib.or_scene_get_camera(self.ctx, scene, _ptr(p), _ptr(d)), "get_camera")
        return p, d

    def frame_setup(self, scene):
        M = np.zeros(16, np.float32)
        P = np.zeros(24, np.float32)
        _chk(self.lib.or_scene_frame_setup(self.ctx, scene, _ptr(M), _ptr(P)), "frame_setup")
        return M.reshape(4, 4), P.reshape(6, 4)

    def canvas(self, width: int, height: int) -> int:
        return _chk(self.lib.or_canvas_new(self.ctx, width, height), "canvas")

    def init_depth(self, canvas, depth: float):
        _chk(self.lib.or_canvas_init_depth(self.ctx, canvas, depth), "init_depth")

    def apply_offset(self, canvas, x: int, y: int):
        _chk(self.lib.or_canvas_apply_offset(self.ctx, canvas, x, y), "apply_offset")

    def resize(self, canvas, w, h):
        _chk(self.lib.or_canvas_resize(self.ctx, canvas, w, h), "resize")

    def clear(self, canvas):
        _chk(self.lib.or_canvas_clear(self.ctx, canvas), "clear")

    def read(self, canvas, width: int, height: int) -> OracleFrame:
        bgra = np.zeros((height, width, 4), np.uint8)
        depth = np.zeros((height, width), np.float32)
        _chk(self.lib.or_canvas_read(self.ctx, canvas, _ptr(bgra), _ptr(depth)), "read")
        return OracleFrame(bgra, depth)

    def write(self, canvas, bgra: np.ndarray, depth: np.ndarray | None):
        bgra = np.ascontiguousarray(bgra, np.uint8)
        d = None if depth is None else np.ascontiguousarray(depth, np.float32)
        _chk(self.lib.or_canvas_write(self.ctx, canvas, _ptr(bgra), _ptr(d)), "write")

    def render(self, scene, canvas) -> int:
        """Returns 0, or the positive error code the reference would have panicked with."""
        rc = self.lib.or_scene_render(self.ctx, scene, canvas)
        return -rc if rc < 0 else 0

    def transparent_tris(self, obj, mesh, count):
        out = np.zeros((count, 9), np.uint32)
        n = _chk(self.lib.or_object_transparent_tris(self.ctx, obj, mesh, _ptr(out), out.size), "transparent_tris")
        return out[:n]

    def draw_triangle_2d(self, canvas, verts, texmap, clip=None) -> int:
        v = np.ascontiguousarray(verts, np.float32).reshape(24)
        c = None if clip is None else np.ascontiguousarray(clip, np.uint64)
        rc = self.lib.or_canvas_draw_triangle_2d(self.ctx, canvas, _ptr(v), texmap, _ptr(c))
        return -rc if rc < 0 else 0
