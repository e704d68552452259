"""Edge values of the draw call's parameters against the oracle (coverage and
depth bit-exact, colour within COLOUR_TOL_LSB):

- canvas sizes that are not multiples of the resolve tile, down to 1x1 and to
  one pixel high or wide (partial tiles, rows that the 16-byte clear stores
  cannot cover);
- the shading exponent at 0, 1, an odd value and negative values (powi's
  binary exponentiation and its final reciprocal, canvas.rs:733-737);
- the maximum of DG_MAX_LIGHTS = 8 lights, also on a micro-triangle frame
  whose small triangles get their light and halfway vectors in the resolve
  pass;
- narrow and wide fields of view."""
import math

import numpy as np
import pytest

from draw_gb300 import scenes as S
from helpers import compare, describe, first_mismatch, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


def _check(desc, gpu_ctx, min_covered=0):
    ref = oracle_render(desc)
    got = gpu_render(desc, gpu_ctx)
    assert got[2] == 0, f"{desc.name}: status {got[2]}"
    p = compare(ref, got, desc.clear_depth)
    assert p.ok, f"{desc.name}: {describe(p)}; {first_mismatch(ref, got)}"
    assert p.n_covered >= min_covered, f"{desc.name}: {describe(p)}"


@pytest.mark.parametrize("w,h", [(1, 1), (3, 5), (37, 23), (31, 33), (1000, 7), (7, 1000), (65, 1), (33, 97)])
def test_canvas_shapes(w, h, gpu_ctx, oracle_lib):
    _check(S.torus_scene(width=w, height=h, nu=40, nv=16, tex=64), gpu_ctx)


@pytest.mark.parametrize("e", [0, 1, 7, -1, -3])
def test_exponents(e, gpu_ctx, oracle_lib):
    _check(S.torus_scene(width=200, height=150, nu=40, nv=16, tex=64, exponent=e), gpu_ctx, min_covered=5000)


def _lights(n, radius=4.0):
    return np.array([[radius * math.cos(2 * math.pi * k / n), 2.0 + 0.5 * k, radius * math.sin(2 * math.pi * k / n)]
                     for k in range(n)], np.float32)


def test_eight_lights(gpu_ctx, oracle_lib):
    desc = S.torus_scene(width=320, height=240, nu=40, nv=16, tex=64, exponent=5)
    desc.lights = _lights(8)
    _check(desc, gpu_ctx, min_covered=10000)


def test_eight_lights_micro_triangles(gpu_ctx, oracle_lib):
    """About 900k vertices and 8 lights make a light/halfway table beyond 128 MB
    on a frame of more triangles than pixels: its small triangles' vectors are
    computed in the resolve pass."""
    desc = S.micro_sphere_field(width=320, height=180, n_tris=1_000_000, tex=64)
    desc.lights = _lights(8, radius=8.0)
    assert desc.n_tris >= desc.width * desc.height
    _check(desc, gpu_ctx, min_covered=10000)


@pytest.mark.parametrize("fov,min_covered", [(5.0, 1000), (20.0, 10000), (120.0, 1000), (175.0, 1)])
def test_fields_of_view(fov, min_covered, gpu_ctx, oracle_lib):
    _check(S.torus_scene(width=240, height=160, nu=40, nv=16, tex=64, fov_x=fov), gpu_ctx, min_covered)
