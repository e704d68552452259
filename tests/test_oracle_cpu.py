"""CPU tests of the oracle: hand-derived known answers for the reference's
rasterization rules, and agreement with the independent pure-Python
restatement (tests/pyref.py) on small seeded scenes."""
import numpy as np
import pytest

import cases
import pyref
from draw_gb300 import scenes as S
from helpers import compare, describe, oracle_render

AZUL_BGRA = (255, 186, 155, 255)


def _screen_tri_scene(pts, width=16, height=12, mats=None, order=None):
    """A scene whose triangles land on the given snapped screen centres.

    World points lie on z = 0 in front of a camera at (0,0,10) looking down -z,
    so screen coordinates are affine in world x and y; the inverse map is
    computed from the oracle's own transformation matrix in float64 and aimed
    0.1 px off the rounding boundary."""
    import oracle

    o = oracle.Oracle()
    s = o.scene(width, height)
    o.set_camera(s, (0.0, 0.0, 10.0), (0.0, 0.0, -10.0), np.float32(width) / np.float32(height), -1.0, -100.0, 60.0)
    M, _ = o.frame_setup(s)
    M = M.astype(np.float64)
    # screen = (M[0]·p / M[3]·p, M[1]·p / M[3]·p) with p = (X, Y, 0, 1) and M[3]·p = -10
    w = M[3, 3]
    world = []
    for sx, sy in pts:
        X = ((sx + 0.1) * w - M[0, 3]) / M[0, 0]
        Y = ((sy + 0.1) * w - M[1, 3]) / M[1, 1]
        world.append([X, Y, 0.0])
    tris = np.arange(len(pts)).reshape(-1, 3)
    mats = mats or [S.Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, -1, -1)]
    split = [(1, i if len(mats) > 1 else 0) for i in range(len(tris))]
    obj = cases._obj(world, tris, mats, mesh_split=split)
    return S.SceneDesc(width, height, cam_pos=(0.0, 0.0, 10.0), cam_dir=(0.0, 0.0, -10.0), near=-1.0, far=-100.0,
                       fov_x=60.0, lights=np.array([[2.0, 3.0, 9.0]], np.float32), exponent=2, textures=[],
                       objects=[obj])


def test_empty_scene_clears(oracle_lib):
    d = S.SceneDesc(20, 10, textures=[], objects=[], clear_depth=100000.0)
    bgra, depth, st = oracle_render(d)
    assert st == 0
    assert (bgra.reshape(-1, 4) == AZUL_BGRA).all()
    assert (depth == np.float32(100000.0)).all()


def test_tie_rule_known_answer(oracle_lib):
    """Right triangle a=(2,2), b=(6,2), c=(2,6): the (-1,-1) tie rule draws the
    hypotenuse x+y=8 (same side as (-1,-1)) but not the legs x=2, y=2, so exactly
    the 6 pixels x>=3, y>=3, x+y<=8 are covered."""
    d = _screen_tri_scene([(2, 2), (6, 2), (2, 6)])
    bgra, depth, st = oracle_render(d)
    assert st == 0
    cov = {(x, y) for y in range(d.height) for x in range(d.width) if np.isfinite(depth[y, x])}
    assert cov == {(3, 3), (3, 4), (3, 5), (4, 3), (4, 4), (5, 3)}
    # colour rows are stored top-down (canvas.rs:941-942)
    for x, y in cov:
        assert tuple(bgra[d.height - 1 - y, x]) != AZUL_BGRA
    assert tuple(bgra[d.height - 1 - 2, 2]) == AZUL_BGRA


def test_tie_rule_reversed_winding_not_culled_twice(oracle_lib):
    """The mirrored triangle (a=(6,6), b=(2,6), c=(6,2)) faces the camera and
    draws the complementary edges: both legs x=6, y=6 (the (-1,-1) side), not the
    hypotenuse."""
    d = _screen_tri_scene([(6, 6), (2, 6), (6, 2)])
    bgra, depth, st = oracle_render(d)
    cov = {(x, y) for y in range(d.height) for x in range(d.width) if np.isfinite(depth[y, x])}
    expect = {(x, y) for x in range(2, 7) for y in range(2, 7) if x + y >= 9}
    assert cov == expect


def test_equal_depth_first_submission_wins(oracle_lib):
    """Two identical triangles with different materials: the strict depth test
    (canvas.rs:923) keeps the first one's colour everywhere."""
    mats = [S.Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, -1, -1),
            S.Material((0.9,) * 3, (0.1,) * 3, (0.6,) * 3, 1.0, -1, -1)]
    both = _screen_tri_scene([(1, 1), (10, 1), (1, 9), (1, 1), (10, 1), (1, 9)], mats=mats)
    first = _screen_tri_scene([(1, 1), (10, 1), (1, 9)], mats=mats[:1])
    second = _screen_tri_scene([(1, 1), (10, 1), (1, 9)], mats=mats[1:])
    b, _, _ = oracle_render(both)
    f1, _, _ = oracle_render(first)
    f2, _, _ = oracle_render(second)
    assert np.array_equal(b, f1)
    assert not np.array_equal(f1, f2)


def test_texture_range_panics(oracle_lib):
    assert oracle_render(cases.texture_range_scene())[2] == 3


def test_reference_default_frame_setup(oracle_lib):
    """Scene::new(800, 600): camera (0,0,150) looking at the origin, so the view
    is a pure translation and M's last row is (0, 0, 1, -150); the x scale is
    (W/2) * (2/(r-l)) * near with r = 10 tan(67.5 deg)."""
    import oracle

    o = oracle.Oracle()
    s = o.scene(800, 600)
    M, P = o.frame_setup(s)
    assert list(M[3]) == [0.0, 0.0, 1.0, -150.0]
    r = 10.0 * np.tan(np.radians(67.5))
    assert M[0, 0] == pytest.approx(400.0 * (1.0 / r) * -10.0, rel=1e-6)
    assert M[0, 1] == 0.0 and M[1, 0] == 0.0
    assert M[0, 2] == pytest.approx(399.5, rel=1e-6)
    # every plane keeps the frustum's interior point on its positive side
    vis = np.array([0.0, 0.0, 150.0 - 100.0])
    for n, k in zip(P[:, :3], P[:, 3]):
        assert float(np.dot(n, vis) + k) > 0


@pytest.mark.parametrize("name", ["tie_rule", "equal_depth", "clip", "degenerate", "offset_collapse"])
def test_pyref_matches_oracle(name, oracle_lib):
    d = cases.PARITY_CASES[name]()
    if name == "offset_collapse":
        d = S.torus_scene(width=160, height=100, nu=16, nv=8, tex=32, exponent=2)
        d.offset, d.canvas_wh, d.clear_depth = (50, 30), (60, 40), 100000.0
    ref = oracle_render(d)
    py = pyref.render(d)
    p = compare(ref, (py[0], py[1]), d.clear_depth)
    assert p.coverage_equal and p.depth_bits_equal and p.colour_max_lsb == 0, describe(p)


def test_pyref_matches_oracle_multilight():
    d = cases.multi_object_scene()
    d.width, d.height = 64, 48
    ref = oracle_render(d)
    py = pyref.render(d)
    p = compare(ref, (py[0], py[1]), d.clear_depth)
    assert p.ok and p.colour_max_lsb == 0 and p.n_covered > 200, describe(p)


def test_pyref_matches_oracle_torus():
    d = S.torus_scene(width=72, height=54, nu=20, nv=8, tex=64, exponent=32)
    ref = oracle_render(d)
    py = pyref.render(d)
    p = compare(ref, (py[0], py[1]), d.clear_depth)
    assert p.ok and p.colour_max_lsb == 0 and p.n_covered > 500, describe(p)


@pytest.mark.parametrize("interp,filt", [(1, 0), (0, 1), (1, 1)])
def test_pyref_matches_oracle_extension_modes(interp, filt):
    """The opt-in extensions (perspective-correct attribute interpolation,
    bilinear texture fetch) restated twice agree bit for bit; coverage and
    depth equal the reference mode's, and the colours differ from it."""
    d = S.torus_scene(width=72, height=54, nu=20, nv=8, tex=64, exponent=32)
    d.cam_pos = (0.3, 1.1, 1.7)
    d.cam_dir = tuple(-c for c in d.cam_pos)
    base = oracle_render(d)
    d.interpolation = interp
    d.textures[0].filter = filt
    ref = oracle_render(d)
    py = pyref.render(d)
    p = compare(ref, (py[0], py[1]), d.clear_depth)
    assert p.ok and p.colour_max_lsb == 0 and p.n_covered > 500, describe(p)
    q = compare(base, (ref[0], ref[1]), d.clear_depth)
    assert q.coverage_equal and q.depth_bits_equal and q.colour_frac_diff > 0.05, describe(q)
