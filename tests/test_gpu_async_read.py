"""dg_canvas_read_async / dg_canvas_read_wait: the copy of a frame overlaps the
next frame's render into another canvas, yields the same bytes as the
synchronous dg_canvas_read, and whatever the context stream does to the canvas
afterwards (a clear, the next render) is ordered after the copy."""
import numpy as np
import pytest
import torch

from draw_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _pinned(h, w):
    bgra = torch.empty((h, w, 4), dtype=torch.uint8, pin_memory=True).numpy()
    depth = torch.empty((h, w), dtype=torch.float32, pin_memory=True).numpy()
    return bgra, depth


def test_async_read_equals_sync_read_and_is_ordered(gpu_ctx):
    from draw_gb300 import renderer

    desc = S.torus_scene(width=320, height=240, tex=64)
    a = renderer.build_scene(desc, gpu_ctx)
    b = renderer.build_scene(desc, gpu_ctx)
    b.scene.camera.reset(tuple(np.float32(c) * np.float32(1.3) for c in desc.cam_pos), desc.cam_dir,
                         float(desc.ratio), desc.near, desc.far, desc.fov_x)
    a.scene.render(a.canvas)
    ref_a = a.canvas.read()
    b.scene.render(b.canvas)
    ref_b = b.canvas.read()
    assert not np.array_equal(ref_a[0], ref_b[0])

    pa, pb = _pinned(240, 320), _pinned(240, 320)
    for _ in range(3):  # a two-canvas pipeline: render, copy out, render the other
        a.scene.render(a.canvas)
        a.canvas.read_async(*pa)
        b.scene.render(b.canvas)
        b.canvas.read_async(*pb)
        a.canvas.clear()  # ordered after a's copy: the copy still holds the rendered frame
        a.canvas.read_wait()
        b.canvas.read_wait()
        assert np.array_equal(pa[0], ref_a[0]) and np.array_equal(pa[1].view(np.uint32), ref_a[1].view(np.uint32))
        assert np.array_equal(pb[0], ref_b[0]) and np.array_equal(pb[1].view(np.uint32), ref_b[1].view(np.uint32))
    cleared = a.canvas.read()[0]
    assert not np.array_equal(cleared, ref_a[0])


def test_read_wait_without_async_read_returns(gpu_ctx):
    from draw_gb300 import renderer

    desc = S.torus_scene(width=64, height=48, tex=16)
    a = renderer.build_scene(desc, gpu_ctx)
    a.canvas.read_wait()
    bgra, _ = _pinned(48, 64)
    a.scene.render(a.canvas)
    a.canvas.read_async(bgra, None)
    a.canvas.read_wait()
    assert np.array_equal(bgra, a.canvas.read(depth=False)[0])


def test_graph_batch_replay_waits_for_pending_copy(gpu_ctx):
    """A graph replay that renders into a canvas with a copy in flight is ordered
    after the copy: the copy holds the frame rendered before the replay."""
    from draw_gb300 import renderer

    frames = S.batch_frames(n_frames=3, seed=17, side_range=(96, 160), tri_range=(2_000, 20_000), tex_range=(64, 64))
    built = [renderer.build_scene(d, gpu_ctx) for d in frames]
    batch = gpu_ctx.batch([b.scene for b in built], [b.canvas for b in built])
    try:
        batch.render()
        refs = [b.canvas.read() for b in built]
        pins = [_pinned(b.canvas.height, b.canvas.width) for b in built]
        for b, p in zip(built, pins):
            b.canvas.read_async(*p)
        for d, b in zip(frames, built):  # move the cameras: the next replay draws different frames
            b.scene.camera.reset(tuple(np.float32(c) * np.float32(1.2) for c in d.cam_pos), d.cam_dir,
                                 float(d.ratio), d.near, d.far, d.fov_x)
        batch.render()
        for b, p, ref in zip(built, pins, refs):
            b.canvas.read_wait()
            assert np.array_equal(p[0], ref[0]) and np.array_equal(p[1].view(np.uint32), ref[1].view(np.uint32))
        moved = [b.canvas.read()[0] for b in built]
        assert any(not np.array_equal(m, r[0]) for m, r in zip(moved, refs))
    finally:
        batch.close()
