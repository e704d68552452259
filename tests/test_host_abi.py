"""CPU tests of the C ABI: the library loads and exports every symbol that
include/draw_gpu.h declares, and its host-side logic (Scene::new defaults,
camera movement, transformation matrix, view planes, argument validation)
matches the oracle bit for bit in a host-only context (device -1)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from draw_gb300 import _build, renderer

    _build.build()
    return renderer.load_library()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "draw_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dg_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    from draw_gb300 import renderer

    syms = header_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(renderer.SIGNATURES), set(syms) - set(renderer.SIGNATURES)


def host_ctx(lib):
    h = ctypes.c_void_p()
    assert lib.dg_ctx_create(-1, ctypes.byref(h)) == 0
    return h


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def frame_setup(lib, h, sid):
    M = np.zeros(16, np.float32)
    P = np.zeros(24, np.float32)
    st = lib.dg_scene_frame_setup(h, sid, _p(M), _p(P))
    return st, M.reshape(4, 4), P.reshape(6, 4)


CAMERAS = [
    ((0.0, 0.0, 150.0), (-0.0, -0.0, -150.0), -10.0, -510.0, 135.0),
    ((0.0, 1.5, 2.598), (0.0, -1.5, -2.598), -0.5, -100.0, 60.0),
    ((3.0, -2.0, 7.0), (-0.3, 0.2, -1.0), -0.05, -60.0, 90.0),
    ((-120.0, 40.0, 10.0), (1.0, -0.1, 0.05), -10.0, -510.0, 170.0),
]


@pytest.mark.parametrize("cam", CAMERAS)
@pytest.mark.parametrize("wh", [(800, 600), (1920, 1080), (257, 129)])
def test_frame_setup_matches_oracle(lib, oracle_lib, cam, wh):
    pos, d, near, far, fov = cam
    h = host_ctx(lib)
    sid = ctypes.c_int32()
    assert lib.dg_scene_create(h, wh[0], wh[1], ctypes.byref(sid)) == 0
    ratio = np.float32(wh[0]) / np.float32(wh[1])
    p, dd = np.array(pos, np.float32), np.array(d, np.float32)
    assert lib.dg_scene_set_camera(h, sid.value, _p(p), _p(dd), ratio, near, far, fov) == 0
    st, M, P = frame_setup(lib, h, sid.value)
    assert st == 0
    o = oracle_lib.Oracle()
    s = o.scene(*wh)
    o.set_camera(s, pos, d, ratio, near, far, fov)
    Mo, Po = o.frame_setup(s)
    assert np.array_equal(M.view(np.uint32), Mo.view(np.uint32))
    assert np.array_equal(P.view(np.uint32), Po.view(np.uint32))
    lib.dg_ctx_destroy(h)


def test_scene_defaults_and_camera_ops_match_oracle(lib, oracle_lib):
    h = host_ctx(lib)
    sid = ctypes.c_int32()
    assert lib.dg_scene_create(h, 800, 600, ctypes.byref(sid)) == 0
    o = oracle_lib.Oracle()
    s = o.scene(800, 600)
    ops = [(3, [5.0]), (0, [2.0]), (6, [10.0]), (2, [1.5]), (4, [3.0]), (5, [1.0]), (1, [0.5]),
           (8, [40.0, -12.0]), (7, [1.0, 2.0, 90.0]), (6, [-33.0])]
    for op, args in ops:
        a = np.zeros(3, np.float32)
        a[: len(args)] = args
        assert lib.dg_scene_camera_op(h, sid.value, op, _p(a)) == 0
        o.camera_op(s, op, args)
        st, M, P = frame_setup(lib, h, sid.value)  # render updates the basis every frame
        Mo, Po = o.frame_setup(s)
        assert st == 0
        assert np.array_equal(M.view(np.uint32), Mo.view(np.uint32)), op
        assert np.array_equal(P.view(np.uint32), Po.view(np.uint32)), op
    pos, d = np.zeros(3, np.float32), np.zeros(3, np.float32)
    assert lib.dg_scene_get_camera(h, sid.value, _p(pos), _p(d)) == 0
    po, do = o.get_camera(s)
    assert np.array_equal(pos.view(np.uint32), po.view(np.uint32))
    assert np.array_equal(d.view(np.uint32), do.view(np.uint32))
    lib.dg_ctx_destroy(h)


def test_camera_assertions_are_status_codes(lib):
    """Camera::new asserts fov < 180, near < 0, near > far (scene/mod.rs:327-331)."""
    h = host_ctx(lib)
    sid = ctypes.c_int32()
    assert lib.dg_scene_create(h, 64, 48, ctypes.byref(sid)) == 0
    p, d = np.array([0, 0, 5], np.float32), np.array([0, 0, -1], np.float32)
    r = np.float32(64 / 48)
    assert lib.dg_scene_set_camera(h, sid.value, _p(p), _p(d), r, -1.0, -100.0, 180.0) == 4
    assert lib.dg_scene_set_camera(h, sid.value, _p(p), _p(d), r, 1.0, -100.0, 60.0) == 4
    assert lib.dg_scene_set_camera(h, sid.value, _p(p), _p(d), r, -10.0, -5.0, 60.0) == 4
    # a camera looking straight up has no basis (u = up x w = 0): the basis assertion fails
    up = np.array([0, 1, 0], np.float32)
    assert lib.dg_scene_set_camera(h, sid.value, _p(p), _p(up), r, -1.0, -100.0, 60.0) == 0
    assert frame_setup(lib, h, sid.value)[0] == 4
    # move_camera_direction asserts dx < width
    a = np.array([64, 0, 0], np.float32)
    assert lib.dg_scene_camera_op(h, sid.value, 8, _p(a)) == 1
    lib.dg_ctx_destroy(h)


def test_host_only_context_refuses_device_work(lib):
    h = host_ctx(lib)
    out = ctypes.c_int32()
    img = np.zeros(12, np.uint8)
    assert lib.dg_texmap_create(h, _p(img), 12, 2, 2, 3, ctypes.byref(out)) == 6
    assert lib.dg_canvas_create(h, 8, 8, ctypes.byref(out)) == 6
    assert lib.dg_ctx_synchronize(h) == 6
    assert lib.dg_scene_create(h, 0, 8, ctypes.byref(out)) == 1
    assert lib.dg_scene_set_lights(h, 0, None, 0) == 1
    assert lib.dg_status_string(3) == b"texel offset outside the texture map"
    assert lib.dg_canvas_read_async(h, 0, None, None) == 1  # no such canvas
    assert lib.dg_canvas_read_wait(h, 0) == 1
    n = ctypes.c_uint64()
    assert lib.dg_check_division(h, 1, 16, 1, ctypes.byref(n), None, None) == 6
    assert lib.dg_check_division(h, 4, 16, 1, ctypes.byref(n), None, None) == 1  # no such sample family
    assert lib.dg_timeline_read(h, None, 4) == 1
    tl = (ctypes.c_uint64 * 20)()
    assert lib.dg_timeline_read(h, tl, 20) == 6  # no device here
    # a graph batch or an autotune run renders each canvas once: a repeated canvas is refused
    ids = (ctypes.c_int32 * 2)(0, 0)
    bp = ctypes.c_void_p()
    assert lib.dg_batch_create(h, ids, ids, 2, ctypes.byref(bp)) == 1
    assert lib.dg_autotune(h, ids, ids, 2, 1, None, None) == 1
    lib.dg_ctx_destroy(h)


def test_tuning_round_trip_and_validation(lib):
    h = host_ctx(lib)
    t = (ctypes.c_uint32 * 7)()
    assert lib.dg_ctx_get_tuning(h, t) == 0
    # small_max_px DG_SMALL_MAX_PX_AUTO and tile_rows 0: chosen per frame and per render job
    assert list(t) == [0xFFFFFFFF, 4, 12, 32, 0, 0, 8]
    good = (0, 1, 64, 2, 7, 16, 256)
    assert lib.dg_ctx_set_tuning(h, (ctypes.c_uint32 * 7)(*good)) == 0
    assert lib.dg_ctx_get_tuning(h, t) == 0 and list(t) == list(good)
    for bad in ((4097, 16, 8, 32, 0, 8, 8), (32, 0, 8, 32, 0, 8, 8), (32, 16, 65, 32, 0, 8, 8),
                (32, 16, 8, 0, 0, 8, 8), (32, 16, 8, 8, 0, 4, 8), (32, 16, 8, 8, 0, 12, 8),
                (32, 16, 8, 8, 0, 64, 8), (32, 16, 8, 8, 0, 8, 0), (32, 16, 8, 8, 0, 8, 257)):
        assert lib.dg_ctx_set_tuning(h, (ctypes.c_uint32 * 7)(*bad)) == 1
    assert lib.dg_ctx_get_tuning(h, t) == 0 and list(t) == list(good)
    auto = (0xFFFFFFFF, 4, 12, 32, 0, 0, 8)
    assert lib.dg_ctx_set_tuning(h, (ctypes.c_uint32 * 7)(*auto)) == 0
    assert lib.dg_ctx_get_tuning(h, t) == 0 and list(t) == list(auto)
    assert lib.dg_ctx_set_tuning(h, None) == 1
    lib.dg_ctx_destroy(h)
