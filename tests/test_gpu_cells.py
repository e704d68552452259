"""The resolve pass's empty-cell path: the setup pass marks every 32x32 pixel
cell that a triangle's bounding box reaches with the frame's epoch, and a tile
whose cell is unmarked gets the clear colour and depth without its visibility
keys being read. These tests move the covered region between frames of one
canvas (cells covered in one frame and empty in the next), under every tile
height, and render one canvas twice in one batched call (a new job: the later
frame overwrites the canvas, as two Scene::render calls do)."""
import numpy as np
import pytest

import cases
from helpers import compare, describe, first_mismatch, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tile_rows", [8, 16, 32])
def test_covered_region_moves_between_frames(tile_rows, gpu_ctx, oracle_lib):
    desc = cases.reference_default_scene(width=256, height=160)
    ops = [(3, (40.0,))]  # Camera::move_right by 40 per frame: the torus slides left
    before = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(tile_rows=tile_rows)
        covered = []
        for frames in (1, 2, 4):
            ref = oracle_render(desc, frames=frames, camera_ops=ops)
            got = gpu_render(desc, gpu_ctx, frames=frames, camera_ops=ops)
            p = compare(ref, got, desc.clear_depth)
            assert p.ok, f"{frames} frames: {describe(p)}; {first_mismatch(ref, got)}"
            covered.append(np.isfinite(got[1]) & (got[1] < desc.clear_depth))
        # the frames cover different pixels, so some cells went from covered to empty
        assert (covered[0] & ~covered[2]).any() and covered[2].any()
    finally:
        gpu_ctx.set_tuning(**before)


def test_batch_with_a_repeated_canvas_renders_in_order(gpu_ctx, oracle_lib):
    from draw_gb300 import renderer

    da, db = cases.small_sphere_field(seed=9), cases.small_sphere_field(seed=10)
    ba, bb = renderer.build_scene(da, gpu_ctx), renderer.build_scene(db, gpu_ctx)
    # frames (a -> canvas A), (b -> canvas A), (a -> canvas B): A ends with b, B with a
    gpu_ctx.render_batch([ba.scene, bb.scene, ba.scene], [ba.canvas, ba.canvas, bb.canvas])
    for canvas, d in ((ba.canvas, db), (bb.canvas, da)):
        got = (*canvas.read(), 0)
        ref = oracle_render(d)
        p = compare(ref, got, d.clear_depth)
        assert p.ok, f"{d.name}: {describe(p)}; {first_mismatch(ref, got)}"
