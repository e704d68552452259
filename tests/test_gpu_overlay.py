"""GPU parity of the 2D overlay triangles (Canvas::draw_triangle,
canvas.rs:435-575): a batch of overlapping, clipped, textured and alpha-blended
triangles drawn over a rendered frame, against the CPU oracle drawing the same
triangles one after the other. Coverage follows the 3D rasterizer's edge
functions and tie rule; colours blend in draw order with the reference's Pixel
arithmetic; only pixels with 0 < depth change."""
import numpy as np
import pytest

import cases
from draw_gb300 import scenes as S
from helpers import compare, describe

pytestmark = pytest.mark.gpu


def _triangles(rng, n, w, h):
    v = np.zeros((n, 3, 8), np.float32)
    v[..., 0] = rng.uniform(-10, w + 10, (n, 3))
    v[..., 1] = rng.uniform(-10, h + 10, (n, 3))
    v[..., 2:4] = rng.uniform(0.0, 0.999, (n, 3, 2))
    v[..., 4:7] = rng.integers(0, 256, (n, 3, 3))
    v[..., 7] = rng.uniform(0.0, 1.2, (n, 3))
    # a few small ones and exact shared edges, as a GUI draw list has
    v[::5, 1:, 0] = v[::5, :1, 0] + rng.integers(1, 6, (len(v[::5]), 2))
    v[1::7, 2, :2] = v[1::7, 0, :2]
    clips = np.stack([rng.integers(0, w // 2, n), rng.integers(0, h // 2, n), rng.integers(w // 2, w, n),
                      rng.integers(h // 2, h, n)], 1).astype(np.uint64)
    return v, clips


@pytest.mark.parametrize("with_clips", [False, True])
def test_overlay_parity(gpu_ctx, oracle_lib, with_clips):
    import oracle

    from draw_gb300 import renderer

    desc = cases.multi_object_scene()
    rng = np.random.default_rng(7)
    tex = S.value_noise_checker(48, 40, 77, comps=4)
    alpha_img = tex.img.reshape(-1, 4).copy()
    alpha_img[:, 3] = rng.integers(0, 256, alpha_img.shape[0])  # varied texel alpha
    verts, clips = _triangles(rng, 120, desc.width, desc.height)

    o = oracle.Oracle()
    texs = [o.texmap(t.img, t.width, t.height, t.comps) for t in desc.textures]
    otm = o.texmap(alpha_img.reshape(-1), tex.width, tex.height, 4)
    s = o.scene(desc.width, desc.height)
    o.set_camera(s, desc.cam_pos, desc.cam_dir, desc.ratio, desc.near, desc.far, desc.fov_x)
    o.set_lights(s, desc.lights)
    o.set_exponent(s, desc.exponent)
    for ob in desc.objects:
        mats = [dict(ka=m.ka, kd=m.kd, ks=m.ks, alpha=m.alpha, map_ka=texs[m.map_ka] if m.map_ka >= 0 else -1,
                     map_kd=texs[m.map_kd] if m.map_kd >= 0 else -1) for m in ob.materials]
        o.add_obj(s, o.object(ob.vertices, ob.normals, ob.uvs, [(m.tris, m.texture_idx) for m in ob.meshes], mats))
    c = o.canvas(desc.width, desc.height)
    o.init_depth(c, desc.clear_depth)
    assert o.render(s, c) == 0
    for t in range(len(verts)):
        assert o.draw_triangle_2d(c, verts[t], otm, clips[t] if with_clips else None) == 0
    ref = o.read(c, desc.width, desc.height)

    b = renderer.build_scene(desc, gpu_ctx)
    tm = renderer.TextureMap(alpha_img.reshape(-1), tex.width, tex.height, 4, gpu_ctx)
    b.scene.render(b.canvas)
    b.canvas.draw_triangles(verts, tm, clips if with_clips else None)
    got = b.canvas.read()
    p = compare((ref.bgra, ref.depth, 0), (*got, 0), desc.clear_depth)
    print(describe(p))
    assert p.ok, describe(p)
    assert int((ref.bgra[..., 3] == 0).sum()) > 500  # pixels the overlay wrote carry padding 0


def test_overlay_texture_range_error(gpu_ctx):
    from draw_gb300 import renderer

    desc = cases.tie_rule_scene()
    b = renderer.build_scene(desc, gpu_ctx)
    tm = renderer.TextureMap(np.full(16 * 16 * 4, 200, np.uint8), 16, 16, 4, gpu_ctx)
    b.scene.render(b.canvas)
    v = np.zeros((1, 3, 8), np.float32)
    v[0, :, :2] = [[2, 2], [40, 3], [5, 30]]
    v[0, :, 2:4] = 2.5  # u, v past 1: the usize offset leaves the image
    v[0, :, 4:7] = 100
    v[0, :, 7] = 1.0
    b.canvas.draw_triangles(v, tm)
    with pytest.raises(renderer.DrawError) as e:
        b.canvas.read()
    assert e.value.status == 3


def test_export_frame_rgba(gpu_ctx, tmp_path):
    """The exported frame is the BGRA frame with bytes 0 and 2 swapped (padding kept as alpha)."""
    from draw_gb300 import imageio, renderer

    desc = cases.multi_object_scene()
    b = renderer.build_scene(desc, gpu_ctx)
    b.scene.render(b.canvas)
    bgra, _ = b.canvas.read()
    rgba = b.canvas.read_rgba()
    assert np.array_equal(rgba[..., 0], bgra[..., 2]) and np.array_equal(rgba[..., 2], bgra[..., 0])
    assert np.array_equal(rgba[..., 1], bgra[..., 1]) and np.array_equal(rgba[..., 3], bgra[..., 3])
    p = str(tmp_path / "frame.png")
    b.canvas.export_frame_as(p)
    img, w, h, c = imageio.read_png(p)
    assert (w, h, c) == (desc.width, desc.height, 4) and np.array_equal(img.reshape(h, w, 4), rgba)
