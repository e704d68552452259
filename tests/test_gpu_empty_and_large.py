"""Empty and maximum-size inputs of the draw call against the oracle
(coverage and depth bit-exact, colour within COLOUR_TOL_LSB):

- a scene without objects, and one whose object has vertices but no
  triangles (Scene::render then only clears: canvas.rs:425-433);
- a batched call that mixes such empty frames with a textured torus;
- a 7680x4320 canvas (33M pixels: job-wide 31-bit pixel indices, 32,400
  resolve tiles, 16-byte clear stores) with the torus in it."""
import numpy as np
import pytest

from draw_gb300 import scenes as S
from helpers import compare, describe, first_mismatch, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


def _empty_object():
    mat = S.Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, 0, 0)
    pos = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], np.float32)
    nrm = np.array([[0.0, 0.0, 1.0]], np.float32)
    uv = np.zeros((1, 3), np.float32)
    return S.ObjectDesc(pos, nrm, uv, [S.MeshDesc(np.zeros((0, 9), np.uint32), 0)], [mat])


def _empty_scenes():
    no_objects = S.SceneDesc(96, 64, textures=[], objects=[], clear_depth=100000.0, name="no_objects")
    tex = S.value_noise_checker(16, 16, 3)
    no_tris = S.SceneDesc(70, 45, textures=[tex], objects=[_empty_object()], name="object_without_triangles")
    return [no_objects, no_tris]


@pytest.mark.parametrize("k", [0, 1])
def test_empty_scene_clears(k, gpu_ctx, oracle_lib):
    desc = _empty_scenes()[k]
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    assert ref[2] == 0 and got[2] == 0
    p = compare(ref, got, desc.clear_depth)
    assert p.ok and p.n_covered == 0, f"{desc.name}: {describe(p)}"


def test_batch_with_empty_frames(gpu_ctx, oracle_lib):
    from draw_gb300 import renderer

    frames = _empty_scenes() + [S.torus_scene(width=160, height=120, nu=40, nv=16, tex=64)]
    built = [renderer.build_scene(d, gpu_ctx) for d in frames]
    gpu_ctx.render_batch([b.scene for b in built], [b.canvas for b in built])
    for d, b in zip(frames, built):
        ref = oracle_render(d)
        got = (*b.canvas.read(), 0)
        p = compare(ref, got, d.clear_depth)
        assert p.ok, f"{d.name}: {describe(p)}; {first_mismatch(ref, got)}"


def test_8k_canvas(gpu_ctx, oracle_lib):
    desc = S.torus_scene(width=7680, height=4320, nu=80, nv=30, tex=512)
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    assert got[2] == 0
    p = compare(ref, got, desc.clear_depth)
    assert p.ok and p.n_covered > 1_000_000, f"{describe(p)}; {first_mismatch(ref, got)}"
