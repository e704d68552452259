"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the same
seeded scenes. Coverage and depth must be bit-exact; colour within
COLOUR_TOL_LSB (1 LSB) per channel, with the differing fraction reported."""
import numpy as np
import pytest

import cases
from draw_gb300 import scenes as S
from helpers import compare, describe, first_mismatch, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(cases.PARITY_CASES))
def test_parity_cases(name, gpu_ctx, oracle_lib):
    desc = cases.PARITY_CASES[name]()
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    assert ref[2] == 0 and got[2] == 0, (ref[2], got[2])
    p = compare(ref, got, desc.clear_depth)
    print(name, describe(p))
    assert p.ok, f"{name}: {describe(p)}; {first_mismatch(ref, got)}"


def test_parity_torus_config(gpu_ctx, oracle_lib):
    """Plain pipeline, CPU-runnable config: torus 4,800 tris, 512^2 RGBA8, 800x600."""
    desc = S.torus_scene()
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    p = compare(ref, got, desc.clear_depth)
    print(describe(p))
    assert p.ok and p.n_covered > 100_000, describe(p)


def test_parity_sphere_field_full(gpu_ctx, oracle_lib):
    """Plain pipeline at scale: 1920x1080, 1M triangles, 2048^2 texture, 2 lights."""
    desc = S.sphere_field()
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    p = compare(ref, got, desc.clear_depth)
    print(describe(p), "near-plane crossing fraction", desc.near_crossing)
    assert p.ok, f"{describe(p)}; {first_mismatch(ref, got)}"


def test_parity_camera_motion(gpu_ctx, oracle_lib):
    """Camera state carried across frames (basis updated inside render)."""
    desc = cases.reference_default_scene()
    ops = [(3, (4.0,)), (0, (2.0,)), (6, (7.0,)), (8, (10, -5))]
    ref = oracle_render(desc, frames=3, camera_ops=ops)
    got = gpu_render(desc, gpu_ctx, frames=3, camera_ops=ops)
    p = compare(ref, got, desc.clear_depth)
    assert p.ok, describe(p)


def test_texture_range_error(gpu_ctx, oracle_lib):
    desc = cases.texture_range_scene()
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    assert ref[2] == 3 and got[2] == 3, (ref[2], got[2])


def test_depth_uninit_error(gpu_ctx):
    from draw_gb300 import renderer

    desc = cases.tie_rule_scene()
    b = renderer.build_scene(desc, gpu_ctx)
    c2 = renderer.Canvas(desc.width, desc.height, gpu_ctx)
    with pytest.raises(renderer.DrawError) as e:
        b.scene.render(c2)
    assert e.value.status == 5


def test_batch_equals_single(gpu_ctx, oracle_lib):
    """The batched form renders every frame exactly as the plain path does."""
    from draw_gb300 import renderer

    frames = S.batch_frames(n_frames=6, seed=77, side_range=(64, 160), tri_range=(500, 20_000), tex_range=(64, 128))
    built = [renderer.build_scene(d, gpu_ctx) for d in frames]
    gpu_ctx.render_batch([b.scene for b in built], [b.canvas for b in built])
    for d, b in zip(frames, built):
        got = (*b.canvas.read(), 0)
        ref = oracle_render(d)
        p = compare(ref, got, d.clear_depth)
        assert p.ok, f"{d.name}: {describe(p)}; {first_mismatch(ref, got)}"


def test_repeat_render_stable(gpu_ctx):
    """Visibility keys are reset by the resolve pass: a second frame is identical."""
    from draw_gb300 import renderer

    desc = cases.small_sphere_field()
    b = renderer.build_scene(desc, gpu_ctx)
    b.scene.render(b.canvas)
    one = b.canvas.read()
    b.scene.render(b.canvas)
    two = b.canvas.read()
    assert np.array_equal(one[0], two[0]) and np.array_equal(one[1].view(np.uint32), two[1].view(np.uint32))


@pytest.mark.parametrize("knobs", [
    dict(small_max_px=0), dict(small_max_px=4096),
    dict(setup_blocks_per_sm=1, queue_blocks_per_sm=1, cull_blocks_per_sm=1),
    dict(small_max_px=256, setup_blocks_per_sm=64, queue_blocks_per_sm=64, cull_blocks_per_sm=64),
    dict(record_limit=1), dict(record_limit=200, small_max_px=0),
    dict(item_units=1, tile_rows=8), dict(item_units=256, tile_rows=16, small_max_px=0)])
def test_tuning_does_not_change_results(knobs, gpu_ctx, oracle_lib):
    """The raster knobs only move work between the in-warp and queue rasterizers,
    resize grids, or (record_limit) send triangles without a record through the
    resolve pass's own setup; coverage, depth and colour stay bit-identical."""
    before = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(**knobs)
        for name in ("torus_strict", "sphere_field_small", "clip"):
            desc = cases.PARITY_CASES[name]()
            ref = oracle_render(desc)
            got = gpu_render(desc, gpu_ctx)
            p = compare(ref, got, desc.clear_depth)
            assert p.ok, f"{name} {knobs}: {describe(p)}; {first_mismatch(ref, got)}"
            st = gpu_ctx.last_stats()
            if knobs.get("record_limit") == 1:
                assert st["triangle_records"] > 1  # some triangles went without a record
    finally:
        gpu_ctx.set_tuning(**before)


def test_parity_stress_config(gpu_ctx, oracle_lib):
    """Stress: 3840x2160, 10M micro-sphere triangles (about 2 px each, depth
    complexity about 8, 10% of the spheres crossing the near plane), 4096^2
    texture, 4 lights; with the default launch shapes and with every small
    triangle on the one-lane-per-triangle path."""
    desc = S.micro_sphere_field()
    ref = oracle_render(desc)
    before = gpu_ctx.get_tuning()
    try:
        for knobs in (dict(), dict(small_max_px=64)):
            gpu_ctx.set_tuning(**knobs)
            got = gpu_render(desc, gpu_ctx)
            p = compare(ref, got, desc.clear_depth)
            print(knobs, describe(p), "near-plane crossing", desc.near_crossing, gpu_ctx.last_stats())
            assert p.ok and p.n_covered > 500_000, f"{knobs}: {describe(p)}; {first_mismatch(ref, got)}"
    finally:
        gpu_ctx.set_tuning(**before)


def test_small_triangle_sorting_keeps_results(gpu_ctx, oracle_lib):
    """Small triangles go to per-lane rasterization in box-size order once there are
    at least 32 per warp of the queue grid (a grid of one block per SM makes a
    200k-triangle micro-sphere field take that path), in plain 32-triangle chunks
    otherwise; both give the oracle's frame."""
    desc = S.micro_sphere_field(width=640, height=360, n_tris=200_000, tex=256, n_lights=2)
    ref = oracle_render(desc)
    before = gpu_ctx.get_tuning()
    try:
        for knobs, sorted_path in ((dict(small_max_px=64, queue_blocks_per_sm=1), True),
                                   (dict(small_max_px=64, queue_blocks_per_sm=64), False)):
            gpu_ctx.set_tuning(**before)
            gpu_ctx.set_tuning(**knobs)
            got = gpu_render(desc, gpu_ctx)
            p = compare(ref, got, desc.clear_depth)
            assert p.ok, f"{knobs}: {describe(p)}; {first_mismatch(ref, got)}"
            import torch

            warps = torch.cuda.get_device_properties(0).multi_processor_count * knobs["queue_blocks_per_sm"] * 8
            assert (gpu_ctx.last_stats()["small_triangles"] >= warps * 32) == sorted_path
    finally:
        gpu_ctx.set_tuning(**before)


def test_clip_deferral_overflow_keeps_results(gpu_ctx, oracle_lib):
    """Survivors that need near-plane clipping are set up in a second pass of each
    setup block, up to 512 per block; beyond that a block clips them in the first
    pass. Micro-spheres that all straddle the near plane, with one setup block per
    SM, exercise both: the frame equals the oracle's."""
    desc = S.micro_sphere_field(width=640, height=360, n_tris=1_000_000, tex=256, n_lights=2, slab=1.0)
    ref = oracle_render(desc)
    before = gpu_ctx.get_tuning()
    try:
        for knobs in (dict(setup_blocks_per_sm=1), dict(setup_blocks_per_sm=16)):
            gpu_ctx.set_tuning(**before)
            gpu_ctx.set_tuning(**knobs)
            got = gpu_render(desc, gpu_ctx)
            p = compare(ref, got, desc.clear_depth)
            assert p.ok, f"{knobs}: {describe(p)}; {first_mismatch(ref, got)}"
            assert gpu_ctx.last_stats()["clip_rows"] > 0
    finally:
        gpu_ctx.set_tuning(**before)


@pytest.mark.parametrize("seed", range(6))
def test_seeded_random_scenes_and_tunings(seed, gpu_ctx, oracle_lib):
    """Seeded variations of the micro-sphere field (sphere size, depth slab, screen
    window, near-plane crossing) rendered under random launch shapes, including a
    record limit that sends some pixels down the record-less path: every frame
    equals the oracle's."""
    rng = np.random.default_rng(1000 + seed)
    desc = S.micro_sphere_field(width=int(rng.choice([320, 480, 640])), height=int(rng.choice([240, 360])),
                                n_tris=int(rng.integers(20_000, 150_000)), seed=int(rng.integers(1, 10_000)),
                                tex=64, n_lights=int(rng.integers(1, 5)), disc_px=float(rng.uniform(1.5, 12.0)),
                                window=float(rng.uniform(0.2, 1.0)), slab=float(rng.uniform(1.0, 30.0)))
    ref = oracle_render(desc)
    knobs = dict(small_max_px=int(rng.choice([0, 4, 16, 64, 256])), item_units=int(rng.choice([1, 4, 8, 32])),
                 setup_blocks_per_sm=int(rng.choice([1, 4, 16])), queue_blocks_per_sm=int(rng.choice([1, 8, 32])),
                 tile_rows=int(rng.choice([8, 16, 32])), record_limit=int(rng.choice([0, 0, 2000])))
    before = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(**knobs)
        got = gpu_render(desc, gpu_ctx)
        p = compare(ref, got, desc.clear_depth)
        assert p.ok, f"{desc.name} {knobs}: {describe(p)}; {first_mismatch(ref, got)}"
    finally:
        gpu_ctx.set_tuning(**before)


def _dense_torus(n_tris=2_200_000, w=200, h=150, lights=4):
    """A frame with more triangles than pixels and a light/halfway table beyond
    128 MB (1.1M vertices x 4 lights x 32 bytes), so DG_FRAME_LAZY: the records
    of its small triangles carry no light rows and the resolve pass computes
    their vertices' light/halfway vectors for the pixels they win."""
    pos, nrm, uv, tri = S.mesh_for_tris("torus", n_tris)
    mat = S.Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, 0, 0)
    cam = (0.4, 1.4, 2.5)
    return S.SceneDesc(w, h, cam_pos=cam, cam_dir=tuple(-c for c in cam), near=-0.5, far=-100.0, fov_x=60.0,
                       lights=np.array([[3.0, 4.0, 3.0], [-2.0, 1.0, 4.0], [0.5, -3.0, 2.0], [-3.0, -2.0, 1.0]][:lights],
                                       np.float32),
                       exponent=5, textures=[S.value_noise_checker(256, 256, 21)],
                       objects=[S.ObjectDesc(pos, nrm, uv, [S.MeshDesc(S._tris9(tri), 0)], [mat])],
                       name=f"dense_torus{n_tris}@{w}x{h}")


def test_parity_dense_frame_lazy_vertex_shading(gpu_ctx, oracle_lib):
    desc = _dense_torus()
    assert desc.n_tris >= desc.width * desc.height
    assert desc.objects[0].vertices.shape[0] * len(desc.lights) * 32 >= 128 << 20
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    p = compare(ref, got, desc.clear_depth)
    assert p.ok and p.n_covered > 5000, f"{describe(p)}; {first_mismatch(ref, got)}"
    # the same frame with the small-triangle path off (every triangle queued): records with rows
    before = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(small_max_px=0)
        got2 = gpu_render(desc, gpu_ctx)
    finally:
        gpu_ctx.set_tuning(**before)
    assert np.array_equal(got[0], got2[0]) and np.array_equal(got[1].view(np.uint32), got2[1].view(np.uint32))
