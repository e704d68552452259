"""The two launch knobs that adapt by themselves when the tuning leaves them at
their defaults (dg_tuning tile_rows 0, small_max_px DG_SMALL_MAX_PX_AUTO):

- the resolve tile height, per render job: the tallest of 32, 16 and 8 rows
  whose tiles fill 4 resolve blocks per SM, else 8;
- the small-triangle threshold, per frame: 64 bounding-box pixels when the
  frame has at least as many triangles as pixels, else 16.

Each case checks the choice (dg_ctx_last_stats entries 12 and 13) and that the
frame equals the oracle's render (coverage and depth bit-exact, colour within
COLOUR_TOL_LSB); fixed knob values override the choice."""
import pytest

from draw_gb300 import scenes as S
from helpers import compare, describe, first_mismatch, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


def _expected_rows(width, height):
    import torch

    slots = 4 * torch.cuda.get_device_properties(0).multi_processor_count
    for rows in (32, 16):
        if ((width + 31) // 32) * ((height + rows - 1) // rows) >= slots:
            return rows
    return 8


CASES = {
    # name: (scene, expected small-triangle threshold)
    "torus_256": (lambda: S.torus_scene(width=256, height=256), 16),
    "torus_800x600": (lambda: S.torus_scene(), 16),
    "torus_1080p": (lambda: S.torus_scene(width=1920, height=1080), 16),
    "micro_320x180": (lambda: S.micro_sphere_field(width=320, height=180, n_tris=100_000, tex=256, n_lights=2), 64),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_adaptive_knobs_choose_and_keep_results(name, gpu_ctx, oracle_lib):
    make, small = CASES[name]
    desc = make()
    assert (desc.n_tris >= desc.width * desc.height) == (small == 64)
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    p = compare(ref, got, desc.clear_depth)
    assert p.ok, f"{name}: {describe(p)}; {first_mismatch(ref, got)}"
    st = gpu_ctx.last_stats()
    assert st["tile_rows"] == _expected_rows(desc.width, desc.height)
    assert st["small_max_px"] == small


def test_fixed_knobs_override_the_choice(gpu_ctx, oracle_lib):
    desc = S.micro_sphere_field(width=320, height=180, n_tris=100_000, tex=256, n_lights=2)
    ref = oracle_render(desc)
    before = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(tile_rows=32, small_max_px=16)
        got = gpu_render(desc, gpu_ctx)
        p = compare(ref, got, desc.clear_depth)
        assert p.ok, f"{describe(p)}; {first_mismatch(ref, got)}"
        st = gpu_ctx.last_stats()
        assert st["tile_rows"] == 32 and st["small_max_px"] == 16
    finally:
        gpu_ctx.set_tuning(**before)
