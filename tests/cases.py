"""Seeded parity cases: small hand-built scenes for the edge cases of the
reference's rasterizer (tie rule, equal-depth ties, clipping branches,
degenerate and NaN geometry, bounding-box collapse, texture range) plus scaled
versions of the benchmark scenes."""
from __future__ import annotations

import math

import numpy as np

from draw_gb300 import scenes as S


def _obj(pos, tris_pos, materials, uvs=None, normals=None, mesh_split=None, tex_idx=None):
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    tp = np.asarray(tris_pos, np.uint32).reshape(-1, 3)
    if uvs is None:
        uvs = np.stack([(pos[:, 0] - pos[:, 0].min()) / max(1e-6, np.ptp(pos[:, 0])),
                        (pos[:, 1] - pos[:, 1].min()) / max(1e-6, np.ptp(pos[:, 1])),
                        np.zeros(len(pos))], 1).astype(np.float32)
    if normals is None:
        normals = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (len(pos), 1))
    tris9 = np.concatenate([tp, tp, tp], 1).astype(np.uint32)
    if mesh_split is None:
        meshes = [S.MeshDesc(tris9, 0 if tex_idx is None else tex_idx)]
    else:
        meshes, start = [], 0
        for n, ti in mesh_split:
            meshes.append(S.MeshDesc(tris9[start:start + n], ti))
            start += n
    return S.ObjectDesc(pos, np.asarray(normals, np.float32), np.asarray(uvs, np.float32), meshes, materials)


def _mat(map_idx=0, ka=0.1, kd=0.7, ks=0.2):
    return S.Material((ka,) * 3, (kd,) * 3, (ks,) * 3, 1.0, map_idx, map_idx)


def flat_scene(objects, width=64, height=48, textures=None, **kw) -> S.SceneDesc:
    """Camera on +z looking at the origin with a narrow fov, so world x/y map to screen x/y."""
    textures = textures if textures is not None else [S.value_noise_checker(64, 64, 7)]
    d = dict(cam_pos=(0.0, 0.0, 10.0), cam_dir=(0.0, 0.0, -10.0), near=-1.0, far=-100.0, fov_x=60.0,
             lights=np.array([[3.0, 4.0, 12.0]], np.float32), exponent=2)
    d.update(kw)
    return S.SceneDesc(width, height, textures=textures, objects=objects, **d)


def tie_rule_scene() -> S.SceneDesc:
    """Right triangles whose axis-aligned legs and shared diagonals pass through
    pixel centres: coverage along them is decided by the (-1,-1) tie rule."""
    objs = []
    pos = [[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0], [-4, -3, 0], [-1, -3, 0], [-4, 0, 0]]
    tris = [[0, 1, 2], [0, 2, 3], [4, 5, 6]]
    objs.append(_obj(pos, tris, [_mat()]))
    return flat_scene(objs)


def equal_depth_scene() -> S.SceneDesc:
    """Coplanar overlapping triangles with different materials: the first
    submission must win every equal-depth pixel (canvas.rs:923 strict <)."""
    pos = [[-3, -2, 0], [3, -2, 0], [0, 3, 0], [-3, -2, 0], [3, -2, 0], [0, 3, 0], [-2, -3, 0], [4, 0, 0], [-1, 2, 0]]
    tris = [[0, 1, 2], [3, 4, 5], [6, 7, 8]]
    mats = [_mat(0, 0.1, 0.7, 0.2), _mat(-1, 0.9, 0.4, 0.5), _mat(0, 0.5, 0.2, 0.9)]
    o = _obj(pos, tris, mats, mesh_split=[(1, 0), (1, 1), (1, 2)])
    o2 = _obj(pos, tris[::-1], mats[::-1], mesh_split=[(1, 0), (1, 1), (1, 2)])
    return flat_scene([o, o2])


def clip_scene(seed=3, n=60) -> S.SceneDesc:
    """Random triangles around the camera's near and far planes: every swap
    branch of ViewPlane::clip and both output cases occur."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = []
    tris = []
    for i in range(n):
        zc = rng.choice([-1.0, -30.0])  # near = -1 around z=9, far = -30 around z=-20 (camera at z=10)
        base = np.array([rng.uniform(-2, 2), rng.uniform(-1.5, 1.5), 10.0 + zc])
        for k in range(3):
            pos.append(base + np.array([rng.uniform(-1.5, 1.5), rng.uniform(-1.5, 1.5), rng.uniform(-3, 3)]))
        tris.append([3 * i, 3 * i + 1, 3 * i + 2])
    pos = np.array(pos, np.float32)
    tris = np.array(tris)
    # face the camera: flip triangles whose normal points away from +z
    a, b, c = pos[tris[:, 0]], pos[tris[:, 1]], pos[tris[:, 2]]
    nz = np.cross(b - a, c - b)[:, 2]
    tris[nz < 0] = tris[nz < 0][:, [0, 2, 1]]
    nrm = np.tile(np.array([[0.2, 0.3, 0.93]], np.float32), (len(pos), 1))
    o = _obj(pos, tris, [_mat()], normals=nrm)
    return flat_scene([o], width=96, height=64, near=-1.0, far=-30.0, fov_x=90.0)


def degenerate_scene() -> S.SceneDesc:
    """Zero-area, repeated-vertex, NaN and huge-coordinate triangles next to a normal one."""
    nan = float("nan")
    pos = [[-2, -2, 0], [2, -2, 0], [0, 2, 0],      # normal
           [-3, 0, 0], [0, 0, 0], [3, 0, 0],        # collinear
           [1, 1, 0], [1, 1, 0], [2, 2, 0],         # repeated vertex
           [nan, 0, 0], [1, 0, 0], [0, 1, 0],       # NaN
           [-1e30, -1, 0], [1e30, -1, 0], [0, 1e30, 0]]  # huge
    tris = [[0, 1, 2], [3, 4, 5], [6, 7, 8], [9, 10, 11], [12, 13, 14]]
    nrm = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (len(pos), 1))
    uvs = np.tile(np.array([[0.5, 0.5, 0.0]], np.float32), (len(pos), 1))
    return flat_scene([_obj(pos, tris, [_mat()], uvs=uvs, normals=nrm)])


def offset_scene() -> S.SceneDesc:
    """The application's setup (app/mod.rs:80-84): the scene is sized to the
    screen and the canvas is a centred window with an offset, so triangles
    outside the canvas hit Rectangle::clip's collapse to column/row 0."""
    d = S.torus_scene(width=320, height=200, nu=40, nv=16, tex=128, exponent=2)
    d.offset = (100, 60)
    d.canvas_wh = (120, 80)  # a 120 x 80 canvas window inside the 320 x 200 scene
    d.clear_depth = 100000.0
    return d


def reference_default_scene(width=200, height=150) -> S.SceneDesc:
    """Scene::new defaults: camera (0,0,150) looking at the origin, fov_x 135,
    near -10, far -510, light (0,300,300), a torus rescaled to radius 100
    like the OBJ loader does (object.rs:159-170), depth cleared to 100000."""
    pos, nrm, uv, tri = S.torus(70.0, 28.0, 48, 20)
    o = S.ObjectDesc(pos, nrm, uv, [S.MeshDesc(S._tris9(tri), 0)],
                     [S.Material((0.9,) * 3, (0.4,) * 3, (0.5,) * 3, 1.0, -1, 0)])
    return S.SceneDesc(width, height, textures=[S.value_noise_checker(256, 256, 11, comps=3)], objects=[o],
                       clear_depth=100000.0)


def multi_object_scene(seed=5) -> S.SceneDesc:
    """Three objects, two materials each, RGB and RGBA maps, default maps, three lights."""
    rng = np.random.Generator(np.random.PCG64(seed))
    texs = [S.value_noise_checker(128, 64, 21, comps=4), S.value_noise_checker(50, 70, 22, comps=3)]
    objs = []
    for i in range(3):
        pos, nrm, uv, tri = S.uv_sphere(0.8, 16, 9, center=tuple(rng.uniform(-1.2, 1.2, 3)))
        t9 = S._tris9(tri)
        half = len(t9) // 2
        mats = [S.Material((0.2,) * 3, (0.6, 0.5, 0.4), (0.3,) * 3, 1.0, i % 2, (i + 1) % 2),
                S.Material((0.9,) * 3, (0.4,) * 3, (0.5,) * 3, 1.5, -1, -1)]
        objs.append(S.ObjectDesc(pos, nrm, uv, [S.MeshDesc(t9[:half], 0), S.MeshDesc(t9[half:], 1)], mats))
    lights = np.array([[3, 4, 5], [-4, 2, 3], [0, -5, 2]], np.float32)
    return S.SceneDesc(160, 120, cam_pos=(0.5, 1.0, 5.0), cam_dir=(-0.5, -1.0, -5.0), near=-0.5, far=-50.0,
                       fov_x=70.0, lights=lights, exponent=5, textures=texs, objects=objs)


def texture_range_scene() -> S.SceneDesc:
    """UVs above 1 make get_rgb_slice's usize subtraction wrap: the reference panics."""
    d = tie_rule_scene()
    d.objects[0].uvs[:, 1] = 3.0
    return d


def small_sphere_field(seed=9, n=40, w=320, h=200) -> S.SceneDesc:
    return S.sphere_field(width=w, height=h, n_spheres=n, slices=20, stacks=11, seed=seed, tex=256, box=8.0)


PARITY_CASES = {
    "tie_rule": tie_rule_scene,
    "equal_depth": equal_depth_scene,
    "clip": clip_scene,
    "degenerate": degenerate_scene,
    "offset_collapse": offset_scene,
    "reference_default": reference_default_scene,
    "multi_object": multi_object_scene,
    "torus_strict": lambda: S.torus_scene(exponent=2),
    "torus_rgb": lambda: S.torus_scene(width=300, height=200, nu=30, nv=12, tex=100, comps=3),
    "sphere_field_small": small_sphere_field,
}


# ------------------------------------------------------------ transparency
def _quad(x0, y0, x1, y1, z):
    """Two triangles facing +z (the flat_scene camera), corners counter-clockwise."""
    return [[x0, y0, z], [x1, y0, z], [x1, y1, z], [x0, y1, z]], [[0, 1, 2], [0, 2, 3]]


def _quads(spec):
    pos, tris = [], []
    for q in spec:
        p, t = _quad(*q)
        tris += [[i + len(pos) for i in tri] for tri in t]
        pos += p
    return pos, tris


def _tmat(alpha, map_idx=0, ka=0.3, kd=0.6, ks=0.25):
    return S.Material((ka,) * 3, (kd, kd * 0.8, kd * 0.6), (ks,) * 3, alpha, map_idx, map_idx)


def transparent_scene() -> S.SceneDesc:
    """Object 0: an opaque quad with two transparent meshes (alpha 0.5 and
    0.25) in front of and behind it; object 1: an opaque quad between object 0's
    transparent layers (drawn after them, it overwrites their blend where it is
    nearer than the opaque quad); object 2: transparent only, in front of
    everything, with a default (white) map."""
    tex = [S.value_noise_checker(64, 64, 31), S.value_noise_checker(32, 48, 32, comps=3)]
    p0, t0 = _quads([(-3, -2, 3, 2, 0.0), (-2.5, -1.5, 1.0, 1.5, 1.0), (-1.0, -1.8, 2.5, 0.5, 2.0),
                     (0.5, -1.0, 3.5, 2.5, 3.0), (-3.5, -2.5, -0.5, 0.5, -1.0), (-2.0, 0.5, 2.8, 2.2, 4.0)])
    o0 = _obj(p0, t0, [_mat(0), _tmat(0.5, 0), _tmat(0.25, 1)], mesh_split=[(2, 0), (6, 1), (4, 2)])
    p1, t1 = _quads([(-1.5, -1.2, 0.8, 0.9, 2.5)])
    o1 = _obj(p1, t1, [_mat(1, ka=0.5, kd=0.4)])
    p2, t2 = _quads([(-2.2, -0.6, 0.2, 1.9, 5.0), (-0.5, -2.4, 1.5, -0.2, 5.5)])
    o2 = _obj(p2, t2, [S.Material((0.2,) * 3, (0.9, 0.3, 0.2), (0.4,) * 3, 0.6, -1, -1)])
    return flat_scene([o0, o1, o2], width=96, height=72, textures=tex)


def transparent_clip_scene() -> S.SceneDesc:
    """Transparent triangles crossing the near plane (both clip outputs), over an opaque torus."""
    pos, nrm, uv, tri = S.torus(1.0, 0.4, 24, 10)
    op = S.ObjectDesc(pos, nrm, uv, [S.MeshDesc(S._tris9(tri), 0)], [_mat(0)])
    rng = np.random.Generator(np.random.PCG64(41))
    tpos = rng.uniform(-2.0, 2.0, (60, 3)).astype(np.float32)
    tpos[:, 2] = rng.uniform(1.0, 3.4, 60).astype(np.float32)  # the camera sits at z = 3, near plane at 2.5
    tt = rng.integers(0, 60, (40, 3)).astype(np.uint32)
    tr = _obj(tpos, tt, [_tmat(0.4, 0), _tmat(0.7, 0)], mesh_split=[(25, 0), (15, 1)])
    return S.SceneDesc(120, 90, cam_pos=(0.0, 0.0, 3.0), cam_dir=(0.0, 0.0, -1.0), near=-0.5, far=-20.0,
                       fov_x=80.0, lights=np.array([[2.0, 3.0, 4.0], [-3.0, 1.0, 2.0]], np.float32), exponent=3,
                       textures=[S.value_noise_checker(64, 64, 43)], objects=[op, tr])


def transparent_ties_scene() -> S.SceneDesc:
    """A transparent mesh whose triangles come in groups of four at exactly equal
    centre distances from any camera on the z axis (rotations by 90 degrees about
    it), so the stable painter's sort must keep the previous frame's order among
    them; plus an opaque backdrop."""
    base = np.array([[1.0, 0.0, 0.0], [2.0, 0.5, 0.0], [1.5, 1.5, 0.0]], np.float32)
    pos, tris = [], []
    for layer, z in enumerate((1.5, 0.5, 1.0)):  # mesh 0: the nearer layer first, so the sort moves it
        for r in range(4):
            c, s = [(1, 0), (0, 1), (-1, 0), (0, -1)][r]
            for v in base:
                pos.append([c * v[0] - s * v[1], s * v[0] + c * v[1], z])
            tris.append([len(pos) - 3, len(pos) - 2, len(pos) - 1])
    tr = _obj(pos, tris, [_tmat(0.5, 0), _tmat(0.3, 0)], mesh_split=[(8, 0), (4, 1)])
    bp, bt = _quads([(-3, -3, 3, 3, -0.5)])
    bg = _obj(bp, bt, [_mat(0)])
    return flat_scene([bg, tr], width=80, height=80, textures=[S.value_noise_checker(32, 32, 51)])


TRANSPARENT_CASES = {
    "transparent": transparent_scene,
    "transparent_clip": transparent_clip_scene,
    "transparent_ties": transparent_ties_scene,
}
