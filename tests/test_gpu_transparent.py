"""GPU parity of the transparent pass (scene/mod.rs:1088-1247): per-mesh
painter's sort kept across frames, no back-face test, near/far clipping, depth
test without depth writes and the Pixel blend, in submission order across
objects. Coverage and depth bit-exact, colour within 1 LSB, against the CPU
oracle; the persistent triangle order equal to the oracle's."""
import numpy as np
import pytest

import cases
from draw_gb300 import scenes as S
from helpers import compare, describe, first_mismatch, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(cases.TRANSPARENT_CASES))
def test_transparent_parity(name, gpu_ctx, oracle_lib):
    desc = cases.TRANSPARENT_CASES[name]()
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    assert ref[2] == 0 and got[2] == 0, (ref[2], got[2])
    p = compare(ref, got, desc.clear_depth)
    blended = int((ref[0][..., 3] == 0).sum())
    print(name, describe(p), "blended pixels", blended)
    assert blended > 100
    assert p.ok, f"{name}: {describe(p)}; {first_mismatch(ref, got)}"


def _oracle_objects(desc):
    import oracle

    o = oracle.Oracle()
    texs = [o.texmap(t.img, t.width, t.height, t.comps) for t in desc.textures]
    s = o.scene(desc.width, desc.height)
    o.set_camera(s, desc.cam_pos, desc.cam_dir, desc.ratio, desc.near, desc.far, desc.fov_x)
    o.set_lights(s, desc.lights)
    o.set_exponent(s, desc.exponent)
    oids = []
    for ob in desc.objects:
        mats = [dict(ka=m.ka, kd=m.kd, ks=m.ks, alpha=m.alpha, map_ka=texs[m.map_ka] if m.map_ka >= 0 else -1,
                     map_kd=texs[m.map_kd] if m.map_kd >= 0 else -1) for m in ob.materials]
        oid = o.object(ob.vertices, ob.normals, ob.uvs, [(m.tris, m.texture_idx) for m in ob.meshes], mats)
        o.add_obj(s, oid)
        oids.append(oid)
    c = o.canvas(*desc.canvas_size)
    o.init_depth(c, desc.clear_depth)
    return o, s, c, oids


@pytest.mark.parametrize("name", ["transparent_ties", "transparent"])
def test_painter_order_persists_across_frames(name, gpu_ctx, oracle_lib):
    """Frames with the camera moving on and off the z axis: after every frame the
    frame and each transparent mesh's triangle order equal the oracle's."""
    from draw_gb300 import renderer

    desc = cases.TRANSPARENT_CASES[name]()
    o, s, c, oids = _oracle_objects(desc)
    b = renderer.build_scene(desc, gpu_ctx)
    moves = [(7, (0.0, 0.0, 10.0)), (7, (0.7, -0.4, 9.0)), (7, (0.0, 0.0, 8.5)), (7, (-1.2, 0.9, 9.5)),
             (7, (0.0, 0.0, 10.0))]
    for op, args in moves:
        o.camera_op(s, op, args)
        b.scene.camera._op(op, *args)
        assert o.render(s, c) == 0
        b.scene.render(b.canvas)
        ref = o.read(c, *desc.canvas_size)
        got = b.canvas.read()
        p = compare((ref.bgra, ref.depth, 0), (*got, 0), desc.clear_depth)
        assert p.ok, f"{args}: {describe(p)}"
        for oi, ob in enumerate(desc.objects):
            nt = [m for m in ob.meshes if ob.materials[m.texture_idx].alpha < 1.0]
            for mi, m in enumerate(nt):
                want = o.transparent_tris(oids[oi], mi, m.tris.shape[0])
                have = b.objects[oi].transparent_triangles(mi)
                assert np.array_equal(want, have), f"object {oi} mesh {mi} after {args}"


def test_batch_with_shared_transparent_object(gpu_ctx, oracle_lib):
    """Two frames of one batch render the same transparent object: the batch
    renders them one after the other, so the second frame sees the order the
    first one left, exactly as two Scene::render calls do."""
    from draw_gb300 import renderer

    desc = cases.transparent_scene()
    b = renderer.build_scene(desc, gpu_ctx)
    s2 = renderer.Scene(desc.width, desc.height, gpu_ctx)
    s2.camera.reset((0.8, -0.5, 9.0), (-0.8, 0.5, -9.0), float(desc.ratio), desc.near, desc.far, desc.fov_x)
    s2.set_lights(desc.lights)
    for ob in b.objects:
        s2.add_obj(ob)
    c2 = renderer.Canvas(desc.width, desc.height, gpu_ctx)
    c2.init_depth(desc.clear_depth)
    gpu_ctx.render_batch([b.scene, s2], [b.canvas, c2])

    o, s, c, oids = _oracle_objects(desc)
    assert o.render(s, c) == 0
    ref1 = o.read(c, *desc.canvas_size)
    o.set_camera(s, (0.8, -0.5, 9.0), (-0.8, 0.5, -9.0), desc.ratio, desc.near, desc.far, desc.fov_x)
    assert o.render(s, c) == 0
    ref2 = o.read(c, *desc.canvas_size)
    for ref, cv in ((ref1, b.canvas), (ref2, c2)):
        got = cv.read()
        p = compare((ref.bgra, ref.depth, 0), (*got, 0), desc.clear_depth)
        assert p.ok, describe(p)


def test_transparent_through_graph_batch(gpu_ctx, oracle_lib):
    """The graph-replayed batch advances the painter's order every replay."""
    from draw_gb300 import renderer

    desc = cases.transparent_ties_scene()
    o, s, c, oids = _oracle_objects(desc)
    b = renderer.build_scene(desc, gpu_ctx)
    g = gpu_ctx.batch([b.scene], [b.canvas])
    try:
        for pos in ((0.0, 0.0, 10.0), (0.5, 0.2, 9.0), (0.0, 0.0, 9.5)):
            o.camera_op(s, 7, pos)
            b.scene.camera._op(7, *pos)
            assert o.render(s, c) == 0
            g.render()
            ref = o.read(c, *desc.canvas_size)
            p = compare((ref.bgra, ref.depth, 0), (*b.canvas.read(), 0), desc.clear_depth)
            assert p.ok, describe(p)
            want = o.transparent_tris(oids[1], 0, 8)
            assert np.array_equal(want, b.objects[1].transparent_triangles(0))
    finally:
        g.close()
