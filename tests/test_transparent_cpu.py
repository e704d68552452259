"""CPU tests of the oracle's transparent pass (scene/mod.rs:1088-1247), pinned
independently of its own transparent code path.

Blend known answer: a quad rendered opaque gives its shaded colour T, the
backdrop alone gives C; rendered with alpha a the quad must give, pixel by
pixel, the reference's Pixel arithmetic (canvas.rs:136-169, 916-921):
  (C * (1 - a)) + (T * a), each product truncated to u8, the sum wrapping,
  the padding byte 0, and the depth buffer untouched.
Painter's sort: triangles at exactly equal centre distances keep their order
(a stable sort), and the order persists between frames."""
import copy

import numpy as np

import cases
from draw_gb300 import scenes as S
from helpers import oracle_render


def _px_mul(p, f):
    """Pixel * f32: (channel as f32 * f) as u8, saturating, NaN -> 0."""
    with np.errstate(invalid="ignore"):
        v = p.astype(np.float32) * np.float32(f)
    v = np.where(np.isnan(v), 0, v)
    return np.clip(np.floor(v), 0, 255).astype(np.uint16)


def _blend(bg, fg, a):
    out = ((_px_mul(bg[..., :3], np.float32(1.0) - np.float32(a)) + _px_mul(fg[..., :3], a)) & 0xFF).astype(np.uint8)
    return np.concatenate([out, np.zeros(out.shape[:-1] + (1,), np.uint8)], -1)


def _scene(alpha, with_quad=True):
    p0, t0 = cases._quads([(-3, -2, 3, 2, 0.0)])
    bg = cases._obj(p0, t0, [cases._mat(0)])
    objs = [bg]
    if with_quad:
        p1, t1 = cases._quads([(-2.0, -1.5, 2.6, 1.0, 1.5), (-3.5, 1.2, -1.0, 2.5, 2.0)])  # disjoint quads
        objs.append(cases._obj(p1, t1, [cases._tmat(alpha, 1)]))
    return cases.flat_scene(objs, width=80, height=60,
                            textures=[S.value_noise_checker(64, 64, 61), S.value_noise_checker(32, 32, 62, comps=3)])


def test_blend_known_answer(oracle_lib):
    C, Cd, st0 = oracle_render(_scene(1.0, with_quad=False))
    T, Td, st1 = oracle_render(_scene(1.0))
    assert st0 == 0 and st1 == 0
    covered = Td.view(np.uint32) != Cd.view(np.uint32)  # pixels of the quads
    assert covered.sum() > 500
    for a in (0.5, 0.25, 0.8, -0.5):
        R, Rd, st = oracle_render(_scene(a))
        assert st == 0
        assert np.array_equal(Rd.view(np.uint32), Cd.view(np.uint32))  # no depth writes
        cov_rows = covered[::-1]  # colour rows are bottom-up relative to depth rows
        exp = np.where(cov_rows[..., None], _blend(C, T, a), C)
        assert np.array_equal(R, exp), f"alpha {a}: {np.argwhere(R != exp)[:3]}"


def test_painter_sort_keeps_ties_and_persists(oracle_lib):
    import oracle

    desc = cases.transparent_ties_scene()
    o = oracle.Oracle()
    texs = [o.texmap(t.img, t.width, t.height, t.comps) for t in desc.textures]
    s = o.scene(desc.width, desc.height)
    o.set_camera(s, desc.cam_pos, desc.cam_dir, desc.ratio, desc.near, desc.far, desc.fov_x)
    o.set_lights(s, desc.lights)
    oids = []
    for ob in desc.objects:
        mats = [dict(ka=m.ka, kd=m.kd, ks=m.ks, alpha=m.alpha, map_ka=texs[m.map_ka] if m.map_ka >= 0 else -1,
                     map_kd=texs[m.map_kd] if m.map_kd >= 0 else -1) for m in ob.materials]
        oid = o.object(ob.vertices, ob.normals, ob.uvs, [(m.tris, m.texture_idx) for m in ob.meshes], mats)
        o.add_obj(s, oid)
        oids.append(oid)
    c = o.canvas(desc.width, desc.height)
    o.init_depth(c, desc.clear_depth)
    before = o.transparent_tris(oids[1], 0, 8)
    o.render(s, c)
    after = o.transparent_tris(oids[1], 0, 8)
    # the camera is on the z axis: the nearer layer (z = 1.5, first in the mesh)
    # sorts after the farther one in descending distance, and within a layer the
    # four equal distances keep their order
    assert np.array_equal(after, np.concatenate([before[4:], before[:4]]))
    o.render(s, c)
    assert np.array_equal(o.transparent_tris(oids[1], 0, 8), after)  # a second frame keeps it
