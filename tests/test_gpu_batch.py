"""GPU tests of the graph-replayed batched form (dg_batch_*) and the launch-shape
autotuner (dg_autotune): every frame of a replay equals the CPU oracle's render
of it (coverage and depth bit-exact, colour within 1 LSB), cameras may move
between replays, shape changes re-capture, and tuning never changes results."""
import numpy as np
import pytest

from draw_gb300 import scenes as S
from helpers import compare, describe, first_mismatch, oracle_render

pytestmark = pytest.mark.gpu


def _frames():
    return S.batch_frames(n_frames=5, seed=91, side_range=(64, 192), tri_range=(500, 30_000), tex_range=(64, 128))


def _check(frames, built):
    for d, b in zip(frames, built):
        got = (*b.canvas.read(), 0)
        ref = oracle_render(d)
        p = compare(ref, got, d.clear_depth)
        assert p.ok, f"{d.name}: {describe(p)}; {first_mismatch(ref, got)}"


def test_graph_batch_equals_oracle_across_replays(gpu_ctx, oracle_lib):
    from draw_gb300 import renderer

    frames = _frames()
    built = [renderer.build_scene(d, gpu_ctx) for d in frames]
    batch = gpu_ctx.batch([b.scene for b in built], [b.canvas for b in built])
    try:
        batch.render()
        batch.render()
        _check(frames, built)
        info = batch.info()
        assert info["captures"] == 1 and info["replays"] == 2 and info["frames"] == len(frames)
        assert info["kernels_per_replay"] == 5
        # moved cameras: the replay uploads new descriptors, no new capture
        for d, b in zip(frames, built):
            d.cam_pos = tuple(np.float32(c) * np.float32(1.25) for c in d.cam_pos)
            b.scene.camera.reset(d.cam_pos, d.cam_dir, float(d.ratio), d.near, d.far, d.fov_x)
        batch.render()
        _check(frames, built)
        assert batch.info()["captures"] == 1
        # a shape change (new tuning) is captured again and renders the same
        before = gpu_ctx.get_tuning()
        try:
            gpu_ctx.set_tuning(small_max_px=0, item_units=2)
            batch.render()
            _check(frames, built)
            assert batch.info()["captures"] == 2
        finally:
            gpu_ctx.set_tuning(**before)
    finally:
        batch.close()


def test_graph_batch_matches_plain_path(gpu_ctx):
    """A replayed batch and one dg_scene_render per frame give identical bytes."""
    from draw_gb300 import renderer

    frames = S.batch_frames(n_frames=12, seed=17, side_range=(128, 320), tri_range=(2_000, 60_000),
                            tex_range=(128, 256))
    built = [renderer.build_scene(d, gpu_ctx) for d in frames]
    for b in built:
        b.scene.render(b.canvas)
    plain = [b.canvas.read() for b in built]
    for b in built:
        b.canvas.clear()
    batch = gpu_ctx.batch([b.scene for b in built], [b.canvas for b in built])
    try:
        for _ in range(3):
            batch.render()
        for (pb, pd), b in zip(plain, built):
            gb, gd = b.canvas.read()
            assert np.array_equal(pb, gb) and np.array_equal(pd.view(np.uint32), gd.view(np.uint32))
    finally:
        batch.close()


def test_batch_config_full_size_equals_oracle(gpu_ctx, oracle_lib):
    """The batching configuration at its stated size, the exact batch bench.py
    times: 256 frames of side 128..512 (log-uniform), meshes of 1k..200k
    triangles, textures 256^2..1024^2 from a pool of 32. Every frame of the
    one-launch-per-stage batch (dg_render_batch) and of its graph replay
    (dg_batch_render) equals the oracle's render of it."""
    from draw_gb300 import renderer
    from helpers import oracle_render_many

    frames = S.batch_frames(n_frames=256, seed=1234)
    assert len(frames) == 256
    refs = oracle_render_many(frames)
    built = [renderer.build_scene(d, gpu_ctx) for d in frames]
    sc, cv = [b.scene for b in built], [b.canvas for b in built]

    def check(tag):
        bad = []
        for d, b, ref in zip(frames, built, refs):
            got = (*b.canvas.read(), 0)
            p = compare(ref, got, d.clear_depth)
            if not p.ok:
                bad.append(f"{tag} {d.name}: {describe(p)}; {first_mismatch(ref, got)}")
        assert not bad, "\n".join(bad[:5]) + f"\n({len(bad)} frames differ)"

    gpu_ctx.render_batch(sc, cv)
    check("render_batch")
    for b in built:
        b.canvas.clear()
    batch = gpu_ctx.batch(sc, cv)
    try:
        batch.render()
        batch.render()
        check("graph replay")
    finally:
        batch.close()


def test_autotune_sets_valid_tuning_and_keeps_results(gpu_ctx, oracle_lib, tmp_path):
    from draw_gb300 import autotune, renderer

    frames = _frames()
    built = [renderer.build_scene(d, gpu_ctx) for d in frames]
    before = gpu_ctx.get_tuning()
    try:
        cache = str(tmp_path / "tuning.json")
        res = autotune.tune(gpu_ctx, [b.scene for b in built], [b.canvas for b in built], reps=2, cache=cache,
                            key="test")
        assert res["ms_per_render"] > 0
        assert gpu_ctx.get_tuning() == res["tuning"]
        gpu_ctx.set_tuning(**before)
        assert autotune.apply(gpu_ctx, cache, "test") == res["tuning"]
        gpu_ctx.render_batch([b.scene for b in built], [b.canvas for b in built])
        _check(frames, built)
    finally:
        gpu_ctx.set_tuning(**before)
