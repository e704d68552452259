"""GPU parity of the two opt-in extensions, which the reference does not have
and which the oracle restates with one fixed expression order each
(oracle/draw_oracle.cpp get_rgb_bilinear and draw_triangle_with_attributes;
tests/pyref.py agrees with it bit for bit):

- perspective-correct interpolation of the shading attributes
  (dg_scene_set_interpolation: DG_INTERP_PERSPECTIVE);
- bilinear texture fetch (dg_texmap_set_filter: DG_FILTER_BILINEAR).

Each mode is checked on the torus configuration and on the full 1920x1080
scene of 1M triangles: coverage and depth bit-exact, colour within
COLOUR_TOL_LSB, and coverage/depth identical to the reference mode's (the
extensions change colours only). Also covered: clipped triangles, transparent
meshes, triangles without a record (shaded from the mesh), the batched and the
graph-replayed forms."""
import numpy as np
import pytest

import cases
from draw_gb300 import scenes as S
from helpers import compare, describe, first_mismatch, gpu_render, oracle_render

pytestmark = pytest.mark.gpu

MODES = [(1, 0), (0, 1), (1, 1)]  # (interpolation, filter)


def _with_modes(desc, interp, filt):
    desc.interpolation = interp
    for t in desc.textures:
        t.filter = filt
    return desc


def _check(desc, gpu_ctx, min_covered=100):
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    assert ref[2] == 0 and got[2] == 0, (ref[2], got[2])
    p = compare(ref, got, desc.clear_depth)
    assert p.ok and p.n_covered >= min_covered, f"{desc.name}: {describe(p)}; {first_mismatch(ref, got)}"
    return ref, got


@pytest.mark.parametrize("interp,filt", MODES)
def test_modes_torus_config(gpu_ctx, oracle_lib, interp, filt):
    base = oracle_render(S.torus_scene())
    ref, _ = _check(_with_modes(S.torus_scene(), interp, filt), gpu_ctx, 100_000)
    q = compare(base, ref)
    assert q.coverage_equal and q.depth_bits_equal and q.colour_frac_diff > 0.01, describe(q)


@pytest.mark.parametrize("interp,filt", MODES)
def test_modes_sphere_field_full(gpu_ctx, oracle_lib, interp, filt):
    _check(_with_modes(S.sphere_field(), interp, filt), gpu_ctx, 100_000)


@pytest.mark.parametrize("name", ["clip", "multi_object", "transparent", "transparent_clip"])
def test_modes_cases(gpu_ctx, oracle_lib, name):
    builders = dict(cases.PARITY_CASES)
    builders.setdefault("transparent", cases.transparent_scene)
    builders.setdefault("transparent_clip", cases.transparent_clip_scene)
    builders.setdefault("multi_object", cases.multi_object_scene)
    _check(_with_modes(builders[name](), 1, 1), gpu_ctx)


def test_modes_without_records(gpu_ctx, oracle_lib):
    """record_limit forces most triangles to be shaded from the mesh in the
    resolve pass (shade_without_record), clipped ones included."""
    before = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(record_limit=7)
        d = _with_modes(cases.PARITY_CASES["clip"](), 1, 1)
        _check(d, gpu_ctx)
        _check(_with_modes(S.torus_scene(width=200, height=150, tex=64), 1, 1), gpu_ctx)
    finally:
        gpu_ctx.set_tuning(**before)


def test_modes_batched_and_graph(gpu_ctx, oracle_lib):
    from draw_gb300 import renderer

    frames = S.batch_frames(n_frames=6, seed=33, side_range=(96, 200), tri_range=(2_000, 30_000), tex_range=(64, 256))
    for i, d in enumerate(frames):
        d.interpolation = i % 2
        d.textures[0] = S.TextureDesc(d.textures[0].img, d.textures[0].width, d.textures[0].height,
                                      d.textures[0].comps, (i // 2) % 2)
    refs = [oracle_render(d) for d in frames]
    built = [renderer.build_scene(d, gpu_ctx) for d in frames]
    sc, cv = [b.scene for b in built], [b.canvas for b in built]
    gpu_ctx.render_batch(sc, cv)
    for d, b, ref in zip(frames, built, refs):
        p = compare(ref, (*b.canvas.read(), 0), d.clear_depth)
        assert p.ok, f"batch {d.name}: {describe(p)}"
    batch = gpu_ctx.batch(sc, cv)
    try:
        batch.render()
        for d, b, ref in zip(frames, built, refs):
            p = compare(ref, (*b.canvas.read(), 0), d.clear_depth)
            assert p.ok, f"graph {d.name}: {describe(p)}"
        # switching a scene back to the reference mode re-captures and renders the reference
        built[1].scene.set_interpolation(0)
        frames[1].interpolation = 0
        batch.render()
        p = compare(oracle_render(frames[1]), (*built[1].canvas.read(), 0), frames[1].clear_depth)
        assert p.ok, describe(p)
    finally:
        batch.close()


def test_mode_arguments_validated(gpu_ctx):
    from draw_gb300 import renderer

    b = renderer.build_scene(S.torus_scene(width=64, height=48, nu=8, nv=4, tex=16), gpu_ctx)
    with pytest.raises(renderer.DrawError):
        b.scene.set_interpolation(2)
    with pytest.raises(renderer.DrawError):
        b.texmaps[0].set_filter(-1)


def test_modes_dense_frame(gpu_ctx, oracle_lib):
    """Both extensions on a frame with more triangles than pixels (lazy vertex
    shading of its small triangles)."""
    from test_gpu_parity import _dense_torus

    _check(_with_modes(_dense_torus(), 1, 1), gpu_ctx, 5000)
