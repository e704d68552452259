"""dg_render_noalloc, the render entry point for callers that cannot allocate
device memory while they draw (a host or plugin that owns a fixed
device-memory budget and lends the renderer only its own buffers, or a frame
loop that must not stall on cudaMalloc/cudaFree, which synchronize the whole
device).

The test calls it through the C ABI, twice in a row on the library's one
shared scratch array, and checks each frame against what the allocating entry
point (dg_scene_render through the Scene/Canvas API) renders for the same scene
and against the CPU oracle: coverage and depth bit-exact, colour within
COLOUR_TOL_LSB. A second test runs a mesh at the triangle limit, with many
triangles across the near plane, then a small mesh after it (the scratch keeps
the large call's contents) on a caller's stream without status_out. The device
buffers for the inputs and outputs are the caller's (allocated here with torch
before the call); the entry point itself allocates nothing.

Kept in a file of its own that pytest collects last, so a run that stops at the
first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from draw_gb300 import scenes as S
from helpers import COLOUR_TOL_LSB, compare, describe, oracle_render

pytestmark = pytest.mark.gpu


def _device_mesh(torch, ob):
    """Uploads an ObjectDesc's arrays in the layout dg_device_mesh describes."""
    nv = ob.vertices.shape[0]
    pos = np.concatenate([ob.vertices, np.ones((nv, 1), np.float32)], 1).astype(np.float32)
    nrm = np.concatenate([ob.normals, np.zeros((ob.normals.shape[0], 1), np.float32)], 1).astype(np.float32)
    uv = np.ascontiguousarray(ob.uvs[:, :2], np.float32)
    tp, tu, tn = [], [], []
    for m in ob.meshes:
        t = np.asarray(m.tris, np.uint32)
        tp.append(np.concatenate([t[:, 0:3], np.full((len(t), 1), m.texture_idx, np.uint32)], 1))
        tu.append(np.concatenate([t[:, 3:6], np.zeros((len(t), 1), np.uint32)], 1))
        tn.append(np.concatenate([t[:, 6:9], np.zeros((len(t), 1), np.uint32)], 1))
    arrs = [pos, nrm, uv] + [np.ascontiguousarray(np.concatenate(x).view(np.int32)) for x in (tp, tu, tn)]
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]
    from draw_gb300.renderer import dg_device_mesh

    m = dg_device_mesh(*[d.data_ptr() for d in dev], nv, ob.normals.shape[0], uv.shape[0], len(np.concatenate(tp)))
    return m, dev


def _device_texmap(torch, t):
    from draw_gb300.renderer import dg_device_texmap

    n = t.img.size
    padded = np.zeros((n + 3) // 4 * 4 + 4, np.uint8)
    padded[:n] = t.img
    d = torch.from_numpy(padded).cuda()
    return dg_device_texmap(d.data_ptr(), n, t.width, t.height, t.comps), d


def _render_noalloc(lib, torch, desc, mesh, texmaps, stream=None, want_status=True):
    from draw_gb300 import renderer as R

    ob = desc.objects[0]
    cw, ch = desc.canvas_size
    p = R.dg_frame_params()
    p.width, p.height, p.canvas_width, p.canvas_height = desc.width, desc.height, cw, ch
    p.cam_pos[:] = list(desc.cam_pos)
    p.cam_dir[:] = list(desc.cam_dir)
    p.near_, p.far_, p.fov_x_deg = desc.near, desc.far, desc.fov_x
    for i, l in enumerate(desc.lights):
        p.lights[i][:] = [float(x) for x in l]
    p.nlights = len(desc.lights)
    p.exponent = desc.exponent
    p.clear_depth = desc.clear_depth
    p.offset_x, p.offset_y = desc.offset
    mats = (R.dg_material * len(ob.materials))()
    for i, m in enumerate(ob.materials):
        mats[i].ka[:], mats[i].kd[:], mats[i].ks[:] = list(m.ka), list(m.kd), list(m.ks)
        mats[i].alpha, mats[i].map_ka, mats[i].map_kd = m.alpha, m.map_ka, m.map_kd
    tex = (R.dg_device_texmap * max(1, len(texmaps)))(*texmaps)
    bgra = torch.zeros(ch * cw * 4, dtype=torch.uint8, device="cuda")
    depth = torch.zeros(ch * cw, dtype=torch.float32, device="cuda")
    status = ctypes.c_int32(-1)
    st = lib.dg_render_noalloc(ctypes.byref(p), ctypes.byref(mesh), ctypes.cast(mats, ctypes.c_void_p),
                               len(ob.materials), ctypes.cast(tex, ctypes.c_void_p), len(texmaps), bgra.data_ptr(),
                               depth.data_ptr(), None if stream is None else ctypes.c_void_p(stream.cuda_stream),
                               ctypes.byref(status) if want_status else None)
    assert st == 0, st
    if want_status:
        assert status.value == 0, status.value
    else:
        stream.synchronize()
    return bgra.cpu().numpy().reshape(ch, cw, 4), depth.cpu().numpy().reshape(ch, cw)


def _render_allocating(gpu_ctx, desc):
    from draw_gb300 import renderer as R

    b = R.build_scene(desc, gpu_ctx)
    b.scene.render(b.canvas)
    return b.canvas.read()


def test_noalloc_matches_allocating_path_twice(gpu_ctx):
    torch = pytest.importorskip("torch")
    from draw_gb300 import renderer as R

    lib = R.load_library()
    first = S.torus_scene(width=256, height=192, nu=40, nv=16, tex=64, exponent=32)
    # second call: same mesh, another camera, exponent, clear value and a canvas window with an offset
    second = S.torus_scene(width=256, height=192, nu=40, nv=16, tex=64, exponent=2, cam_dist=2.7)
    second.cam_pos = (1.2, 0.9, 2.2)
    second.cam_dir = tuple(-c for c in second.cam_pos)
    second.canvas_wh, second.offset, second.clear_depth = (200, 150), (28, 21), 100000.0
    mesh, keep = _device_mesh(torch, first.objects[0])
    texmaps, keep_t = zip(*[_device_texmap(torch, t) for t in first.textures])
    for desc in (first, second):
        got = _render_noalloc(lib, torch, desc, mesh, list(texmaps))
        ref = _render_allocating(gpu_ctx, desc)
        p = compare(ref, got, desc.clear_depth)
        assert p.ok and p.colour_max_lsb <= COLOUR_TOL_LSB and p.n_covered > 1000, describe(p)
        q = compare(oracle_render(desc), got, desc.clear_depth)
        assert q.ok and q.colour_max_lsb <= COLOUR_TOL_LSB, describe(q)


def test_noalloc_at_its_limits_then_small_on_a_stream(gpu_ctx, oracle_lib):
    """A torus of 64,512 triangles (32,637 vertices, within the 65,536 / 32,768
    limits) on a 512x512 canvas (the pixel limit), seen from above with the near
    plane slicing its top (about a thousand triangles cross it); then a small mesh rendered after
    it on a non-default stream with status_out NULL, the caller synchronizing
    the stream. Both frames equal the allocating path's and the oracle's."""
    torch = pytest.importorskip("torch")
    from draw_gb300 import renderer as R

    lib = R.load_library()
    big = S.torus_scene(width=512, height=512, nu=252, nv=128, tex=64, exponent=2)
    big.cam_pos = (0.0, 1.2, 0.0)
    big.cam_dir = (0.05, -1.0, 0.02)
    big.near, big.far = -1.15, -50.0
    assert big.n_tris == 64_512 and big.objects[0].vertices.shape[0] <= 32_768
    small = S.torus_scene(width=160, height=120, nu=12, nv=6, tex=32, exponent=5)
    stream = torch.cuda.Stream()
    for desc, kw in ((big, {}), (small, dict(stream=stream, want_status=False))):
        mesh, keep = _device_mesh(torch, desc.objects[0])
        texmaps, keep_t = zip(*[_device_texmap(torch, t) for t in desc.textures])
        got = _render_noalloc(lib, torch, desc, mesh, list(texmaps), **kw)
        ref = _render_allocating(gpu_ctx, desc)
        p = compare(ref, got, desc.clear_depth)
        assert p.ok and p.n_covered > 1000, describe(p)
        q = compare(oracle_render(desc), got, desc.clear_depth)
        assert q.ok, describe(q)


def test_noalloc_rejects_sizes_beyond_its_limits(gpu_ctx):
    torch = pytest.importorskip("torch")
    from draw_gb300 import renderer as R

    lib = R.load_library()
    desc = S.torus_scene(width=1024, height=512, nu=8, nv=4, tex=16)
    mesh, keep = _device_mesh(torch, desc.objects[0])
    p = R.dg_frame_params()
    p.width, p.height, p.canvas_width, p.canvas_height = 1024, 512, 1024, 512  # 524,288 pixels > 262,144
    p.cam_pos[:] = [0.0, 0.0, 3.0]
    p.cam_dir[:] = [0.0, 0.0, -1.0]
    p.near_, p.far_, p.fov_x_deg, p.nlights, p.clear_depth = -0.5, -100.0, 60.0, 1, float("inf")
    mats = (R.dg_material * 1)()
    mats[0].alpha, mats[0].map_ka, mats[0].map_kd = 1.0, -1, -1
    out = torch.zeros(16, dtype=torch.float32, device="cuda")
    st = lib.dg_render_noalloc(ctypes.byref(p), ctypes.byref(mesh), ctypes.cast(mats, ctypes.c_void_p), 1, None, 0,
                               out.data_ptr(), out.data_ptr(), None, None)
    assert st == 8  # DG_E_LIMIT
