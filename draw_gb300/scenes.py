"""Seeded synthetic scenes for the draw rasterization path.

The reference renders OBJ models; the workloads here are synthetic stand-ins
with the shapes and sizes of the project's benchmark configurations: a textured
torus, fields of UV spheres, mixed-size frame batches and request streams.
Every scene is described by a plain ``SceneDesc`` that both the GPU renderer
(``draw_gb300.renderer``) and the CPU oracle consume, so both see identical
bytes.

Texture noise uses integer hashing only, so textures are bit-identical on every
platform. Geometry uses float64 trigonometry rounded to float32.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Material:
    """The reference's per-mesh `Texture` (scene/mod.rs:206-216). map_* index
    SceneDesc.textures, or -1 for the 1x1 white default map."""

    ka: tuple = (0.1, 0.1, 0.1)
    kd: tuple = (0.7, 0.7, 0.7)
    ks: tuple = (0.2, 0.2, 0.2)
    alpha: float = 1.0
    map_ka: int = -1
    map_kd: int = -1


@dataclass
class MeshDesc:
    tris: np.ndarray  # (T, 9) uint32: position[3], texture[3], normal[3]
    texture_idx: int = 0


@dataclass
class ObjectDesc:
    vertices: np.ndarray  # (V, 3) float32
    normals: np.ndarray  # (N, 3) float32
    uvs: np.ndarray  # (U, 3) float32 (the reference keeps UVs as Vec3 with z = 0)
    meshes: list
    materials: list

    @property
    def n_tris(self) -> int:
        return int(sum(m.tris.shape[0] for m in self.meshes))


@dataclass
class TextureDesc:
    img: np.ndarray  # (H*W*C,) uint8, row 0 = top (stb layout, scene/mod.rs:144)
    width: int
    height: int
    comps: int
    filter: int = 0  # extension: 0 = nearest texel (the reference), 1 = bilinear


@dataclass
class SceneDesc:
    width: int
    height: int
    cam_pos: tuple = (0.0, 0.0, 150.0)
    cam_dir: tuple = (-0.0, -0.0, -150.0)
    near: float = -10.0
    far: float = -510.0
    fov_x: float = 135.0
    lights: np.ndarray = field(default_factory=lambda: np.array([[0.0, 300.0, 300.0]], np.float32))
    exponent: int = 2
    clear_depth: float = float("inf")
    offset: tuple = (0, 0)
    canvas_wh: tuple | None = None  # canvas size when it differs from the scene's (app/mod.rs:58-69)
    interpolation: int = 0  # extension: 0 = screen-space (the reference), 1 = perspective-correct
    textures: list = field(default_factory=list)
    objects: list = field(default_factory=list)
    name: str = ""

    @property
    def n_tris(self) -> int:
        return int(sum(o.n_tris for o in self.objects))

    @property
    def canvas_size(self) -> tuple:
        return tuple(self.canvas_wh) if self.canvas_wh else (self.width, self.height)

    @property
    def ratio(self) -> np.float32:
        return np.float32(self.width) / np.float32(self.height)


# ---------------------------------------------------------------- textures
def _hash2(x: np.ndarray, y: np.ndarray, seed: int) -> np.ndarray:
    """32-bit integer hash of lattice points (a splitmix-style finaliser)."""
    h = (x.astype(np.uint64) * np.uint64(0x9E3779B1) + y.astype(np.uint64) * np.uint64(0x85EBCA77)
         + np.uint64(seed & 0xFFFFFFFF) * np.uint64(0xC2B2AE3D)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x2C1B3C6D)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(12)
    h = (h * np.uint64(0x297A2D39)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    return h


def value_noise_checker(width: int, height: int, seed: int, comps: int = 4, cell: int = 32,
                        check: int = 16) -> TextureDesc:
    """Checkerboard modulated by bilinear value noise, integer arithmetic only."""
    ys, xs = np.meshgrid(np.arange(height, dtype=np.int64), np.arange(width, dtype=np.int64), indexing="ij")
    cx, cy = xs // cell, ys // cell
    fx, fy = xs % cell, ys % cell
    v00 = (_hash2(cx, cy, seed) & np.uint64(255)).astype(np.int64)
    v10 = (_hash2(cx + 1, cy, seed) & np.uint64(255)).astype(np.int64)
    v01 = (_hash2(cx, cy + 1, seed) & np.uint64(255)).astype(np.int64)
    v11 = (_hash2(cx + 1, cy + 1, seed) & np.uint64(255)).astype(np.int64)
    top = v00 * (cell - fx) + v10 * fx
    bot = v01 * (cell - fx) + v11 * fx
    noise = (top * (cell - fy) + bot * fy) // (cell * cell)  # 0..255
    checker = ((xs // check + ys // check) & 1).astype(np.int64)
    base = [(230, 120, 40), (40, 110, 220)]
    img = np.zeros((height, width, comps), np.uint8)
    for ch in range(3):
        b0, b1 = base[0][ch], base[1][ch]
        bch = np.where(checker == 1, b1, b0)
        img[..., ch] = np.clip((bch * (96 + noise)) // 351, 0, 255).astype(np.uint8)
    if comps == 4:
        img[..., 3] = 255
    return TextureDesc(img.reshape(-1), width, height, comps)


# ---------------------------------------------------------------- meshes
def torus(R: float = 1.0, r: float = 0.4, nu: int = 80, nv: int = 30, center=(0.0, 0.0, 0.0)):
    """Seam-duplicated (nu+1) x (nv+1) grid, 2*nu*nv triangles, analytic normals,
    UV = (i/nu, j/nv). Winding is counter-clockwise seen from outside, so the
    reference's back-face test keeps the faces that point at the camera."""
    i = np.arange(nu + 1, dtype=np.float64)
    j = np.arange(nv + 1, dtype=np.float64)
    u = 2.0 * math.pi * i / nu
    v = 2.0 * math.pi * j / nv
    U, Vv = np.meshgrid(u, v, indexing="ij")
    x = (R + r * np.cos(Vv)) * np.cos(U) + center[0]
    y = r * np.sin(Vv) + center[1]
    z = (R + r * np.cos(Vv)) * np.sin(U) + center[2]
    nx = np.cos(Vv) * np.cos(U)
    ny = np.sin(Vv)
    nz = np.cos(Vv) * np.sin(U)
    pos = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float32)
    nrm = np.stack([nx, ny, nz], -1).reshape(-1, 3).astype(np.float32)
    I, J = np.meshgrid(np.arange(nu + 1), np.arange(nv + 1), indexing="ij")
    uv = np.stack([I / nu, J / nv, np.zeros_like(I, dtype=np.float64)], -1).reshape(-1, 3).astype(np.float32)
    idx = lambda a, b: a * (nv + 1) + b  # noqa: E731
    ii, jj = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    ii, jj = ii.reshape(-1), jj.reshape(-1)
    p00, p10, p01, p11 = idx(ii, jj), idx(ii + 1, jj), idx(ii, jj + 1), idx(ii + 1, jj + 1)
    t1 = np.stack([p00, p01, p11], -1)
    t2 = np.stack([p00, p11, p10], -1)
    tri = np.stack([t1, t2], 1).reshape(-1, 3).astype(np.uint32)
    return pos, nrm, uv, _fix_winding(pos, nrm, tri)


def uv_sphere(radius: float = 1.0, slices: int = 50, stacks: int = 21, center=(0.0, 0.0, 0.0)):
    """UV sphere with 2*slices*(stacks-1) triangles (poles as single triangles)."""
    s = np.arange(slices + 1, dtype=np.float64)
    k = np.arange(stacks + 1, dtype=np.float64)
    phi = 2.0 * math.pi * s / slices
    th = math.pi * k / stacks
    P, T = np.meshgrid(phi, th, indexing="ij")
    nx = np.sin(T) * np.cos(P)
    ny = np.cos(T)
    nz = np.sin(T) * np.sin(P)
    pos = (np.stack([nx, ny, nz], -1) * radius + np.asarray(center)).reshape(-1, 3).astype(np.float32)
    nrm = np.stack([nx, ny, nz], -1).reshape(-1, 3).astype(np.float32)
    S_, K_ = np.meshgrid(np.arange(slices + 1), np.arange(stacks + 1), indexing="ij")
    uv = np.stack([S_ / slices, 1.0 - K_ / stacks, np.zeros_like(S_, dtype=np.float64)], -1)
    uv = uv.reshape(-1, 3).astype(np.float32)
    idx = lambda a, b: a * (stacks + 1) + b  # noqa: E731
    tris = []
    ss, kk = np.meshgrid(np.arange(slices), np.arange(stacks), indexing="ij")
    ss, kk = ss.reshape(-1), kk.reshape(-1)
    a, b, c, d = idx(ss, kk), idx(ss + 1, kk), idx(ss, kk + 1), idx(ss + 1, kk + 1)
    top = kk == 0
    bottom = kk == stacks - 1
    mid = ~(top | bottom)
    tris.append(np.stack([a[top], c[top], d[top]], -1))
    tris.append(np.stack([a[mid], c[mid], d[mid]], -1))
    tris.append(np.stack([a[mid], d[mid], b[mid]], -1))
    tris.append(np.stack([a[bottom], c[bottom], b[bottom]], -1))
    tri = np.concatenate(tris).astype(np.uint32)
    return pos, nrm, uv, _fix_winding(pos, nrm, tri)


def _fix_winding(pos, nrm, tri):
    """Orients each triangle so (b-a)x(c-b) agrees with its vertex normals."""
    a, b, c = pos[tri[:, 0]].astype(np.float64), pos[tri[:, 1]].astype(np.float64), pos[tri[:, 2]].astype(np.float64)
    n = np.cross(b - a, c - b)
    s = (n * (nrm[tri[:, 0]] + nrm[tri[:, 1]] + nrm[tri[:, 2]])).sum(-1)
    flip = s < 0
    out = tri.copy()
    out[flip, 1], out[flip, 2] = tri[flip, 2], tri[flip, 1]
    return out


def _tris9(tri: np.ndarray) -> np.ndarray:
    """Position, texture and normal index triples are the same grid index here."""
    return np.ascontiguousarray(np.concatenate([tri, tri, tri], axis=1), dtype=np.uint32)


def _look_at_dir(pos, target):
    return tuple(float(t - p) for p, t in zip(pos, target))


# ---------------------------------------------------------------- configs
def torus_scene(width=800, height=600, seed=1234, nu=80, nv=30, tex=512, exponent=32, cam_dist=3.0,
                fov_x=60.0, comps=4) -> SceneDesc:
    """Plain pipeline, CPU-runnable: torus R=1.0 r=0.4, 80x30 segments (4,800 tris),
    512x512 RGBA8 value-noise checker, 800x600, camera at distance 3, fov 60."""
    pos, nrm, uv, tri = torus(1.0, 0.4, nu, nv)
    t = value_noise_checker(tex, tex, seed, comps=comps)
    mat = Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, 0, 0)
    obj = ObjectDesc(pos, nrm, uv, [MeshDesc(_tris9(tri), 0)], [mat])
    el = math.radians(30.0)
    cam = (0.0, cam_dist * math.sin(el), cam_dist * math.cos(el))
    return SceneDesc(width, height, cam_pos=cam, cam_dir=_look_at_dir(cam, (0, 0, 0)), near=-0.5, far=-100.0,
                     fov_x=fov_x, lights=np.array([[2.0, 4.0, 3.0]], np.float32), exponent=exponent,
                     clear_depth=float("inf"), textures=[t], objects=[obj], name=f"torus{2 * nu * nv}@{width}x{height}")


def sphere_field(width=1920, height=1080, n_spheres=500, slices=50, stacks=21, seed=1234, tex=2048, box=20.0,
                 n_lights=2, near=-0.05, far=-60.0, fov_x=60.0, rmin=0.2, rmax=1.0, exponent=2) -> SceneDesc:
    """Plain pipeline at scale: n_spheres seeded UV spheres (radius U[rmin,rmax],
    centres uniform in a box^3 cube) flattened into one object, camera at the
    cube's centre so about 5% of the instances cross the near plane."""
    rng = np.random.Generator(np.random.PCG64(seed))
    radii = rng.uniform(rmin, rmax, n_spheres)
    centres = rng.uniform(-box / 2, box / 2, (n_spheres, 3))
    base_pos, base_nrm, base_uv, base_tri = uv_sphere(1.0, slices, stacks)
    nvtx = base_pos.shape[0]
    pos = (base_pos[None].astype(np.float64) * radii[:, None, None] + centres[:, None, :]).reshape(-1, 3)
    pos = pos.astype(np.float32)
    nrm = np.tile(base_nrm, (n_spheres, 1))
    uv = np.tile(base_uv, (n_spheres, 1))
    tri = (base_tri[None].astype(np.int64) + (np.arange(n_spheres) * nvtx)[:, None, None]).reshape(-1, 3)
    t = value_noise_checker(tex, tex, seed, comps=4)
    mat = Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, 0, 0)
    obj = ObjectDesc(pos, nrm, uv, [MeshDesc(_tris9(tri.astype(np.uint32)), 0)], [mat])
    cam = (0.0, 0.0, 0.0)
    cdir = (0.3, -0.2, -1.0)
    lights = np.array([[8.0, 9.0, 6.0], [-9.0, 4.0, -7.0], [5.0, -8.0, -9.0], [-6.0, -7.0, 8.0]], np.float32)[:n_lights]
    d = SceneDesc(width, height, cam_pos=cam, cam_dir=cdir, near=near, far=far, fov_x=fov_x, lights=lights,
                  exponent=exponent, clear_depth=float("inf"), textures=[t], objects=[obj],
                  name=f"spheres{n_spheres}x{2 * slices * (stacks - 1)}@{width}x{height}")
    d.near_crossing = near_plane_crossing_fraction(d, centres, radii)
    return d


def micro_sphere_field(width=3840, height=2160, n_tris=10_000_000, slices=5, stacks=5, seed=1234, tex=4096,
                       n_lights=4, fov_x=60.0, near_dist=1.0, disc_px=3.6, window=0.4, slab=20.0,
                       exponent=2) -> SceneDesc:
    """Stress config: n_tris small triangles as seeded micro UV spheres of
    2*slices*(stacks-1) triangles each, flattened into one object.

    Every sphere has the same world radius, chosen so its projected disc at the
    near plane has a radius of about disc_px pixels (about 2 px per triangle);
    centres lie in a slab of depth slab * radius that starts one radius in front
    of the near plane, so about 2/slab of the spheres (10% for slab=20) cross
    it; their screen positions are uniform in a centred window covering
    window^2 of the screen, which sets the depth complexity (about 8 for the
    defaults). The statistics actually reached are stored on the description
    (near_crossing, depth_complexity_est, mean_tri_px_est)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    base_pos, base_nrm, base_uv, base_tri = uv_sphere(1.0, slices, stacks)
    per = base_tri.shape[0]
    n_spheres = max(1, n_tris // per)
    f = (width / 2.0) / math.tan(math.radians(fov_x) / 2.0)  # focal length in pixels
    r = disc_px * near_dist / f
    d = rng.uniform(near_dist - r, near_dist - r + slab * r, n_spheres)  # distance along the view axis
    sx = rng.uniform(-0.5, 0.5, n_spheres) * window * width
    sy = rng.uniform(-0.5, 0.5, n_spheres) * window * height
    centres = np.stack([sx * d / f, sy * d / f, -d], -1)
    nvtx = base_pos.shape[0]
    pos = (base_pos[None].astype(np.float64) * r + centres[:, None, :]).reshape(-1, 3).astype(np.float32)
    nrm = np.tile(base_nrm, (n_spheres, 1))
    uv = np.tile(base_uv, (n_spheres, 1))
    tri = (base_tri[None].astype(np.int64) + (np.arange(n_spheres) * nvtx)[:, None, None]).reshape(-1, 3)
    t = value_noise_checker(tex, tex, seed, comps=4)
    mat = Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, 0, 0)
    obj = ObjectDesc(pos, nrm, uv, [MeshDesc(_tris9(tri.astype(np.uint32)), 0)], [mat])
    lights = np.array([[0.5, 0.8, 0.5], [-0.6, 0.4, -0.2], [0.4, -0.7, -0.3], [-0.5, -0.5, 0.6]],
                      np.float32)[:n_lights]
    desc = SceneDesc(width, height, cam_pos=(0.0, 0.0, 0.0), cam_dir=(0.0, 0.0, -1.0), near=-near_dist,
                     far=-100.0, fov_x=fov_x, lights=lights, exponent=exponent, clear_depth=float("inf"),
                     textures=[t], objects=[obj], name=f"microspheres{n_spheres}x{per}@{width}x{height}")
    desc.near_crossing = float(np.mean(np.abs(d - near_dist) < r))
    disc = math.pi * (disc_px * near_dist / d) ** 2  # projected disc area of each sphere, pixels
    desc.depth_complexity_est = float(disc.sum() / (window * width * window * height))
    desc.mean_tri_px_est = float(disc.mean() / (per / 2.0))  # front-facing half of the triangles
    return desc


def near_plane_crossing_fraction(d: SceneDesc, centres: np.ndarray, radii: np.ndarray) -> float:
    """Fraction of sphere instances that intersect the (infinite) near plane."""
    g = np.asarray(d.cam_dir, np.float64)
    g = g / np.linalg.norm(g)
    p0 = np.asarray(d.cam_pos, np.float64) + g * abs(d.near)
    dist = (centres - p0) @ g
    return float(np.mean(np.abs(dist) < radii))


def mesh_for_tris(kind: str, n_tris: int, radius: float = 1.0):
    """A torus or UV sphere with about n_tris triangles."""
    if kind == "torus":
        nv = max(3, int(round(math.sqrt(n_tris / 2 / 2.7))))
        nu = max(3, int(round(n_tris / 2 / nv)))
        return torus(radius, 0.4 * radius, nu, nv)
    stacks = max(3, int(round(math.sqrt(n_tris / 4)))) + 1
    slices = max(3, int(round(n_tris / (2 * (stacks - 1)))))
    return uv_sphere(radius, slices, stacks)


def random_frame(rng: np.random.Generator, width: int, height: int, n_tris: int, tex_side: int, seed: int,
                 kind: str | None = None, texture: TextureDesc | None = None) -> SceneDesc:
    """One frame of a batch: its own mesh, camera and texture."""
    kind = kind or ("torus" if rng.random() < 0.5 else "sphere")
    pos, nrm, uv, tri = mesh_for_tris(kind, n_tris)
    t = texture if texture is not None else value_noise_checker(tex_side, tex_side, seed, comps=4)
    mat = Material((0.1,) * 3, (0.7,) * 3, (0.2,) * 3, 1.0, 0, 0)
    obj = ObjectDesc(pos, nrm, uv, [MeshDesc(_tris9(tri), 0)], [mat])
    az = rng.uniform(0, 2 * math.pi)
    el = rng.uniform(0.2, 1.0)
    dist = rng.uniform(2.6, 4.0)
    cam = (dist * math.cos(el) * math.sin(az), dist * math.sin(el), dist * math.cos(el) * math.cos(az))
    light = np.array([[3.0 * math.sin(az + 1), 4.0, 3.0 * math.cos(az + 1)]], np.float32)
    return SceneDesc(width, height, cam_pos=cam, cam_dir=_look_at_dir(cam, (0, 0, 0)), near=-0.5, far=-100.0,
                     fov_x=60.0, lights=light, exponent=2, clear_depth=float("inf"), textures=[t],
                     objects=[obj], name=f"{kind}{tri.shape[0]}@{width}x{height}")


def batch_frames(n_frames=256, seed=1234, side_range=(128, 512), tri_range=(1_000, 200_000),
                 tex_range=(256, 1024), tex_pool: int = 32) -> list:
    """Batching workload: square frames of side log-uniform in side_range, meshes
    of log-uniform triangle count in tri_range, textures of side in tex_range.
    Textures come from a seeded pool of tex_pool maps (shared between frames)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pool: dict = {}
    frames = []
    for i in range(n_frames):
        side = int(round(math.exp(rng.uniform(math.log(side_range[0]), math.log(side_range[1])))))
        ntri = int(round(math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))))
        tex = int(2 ** round(rng.uniform(math.log2(tex_range[0]), math.log2(tex_range[1]))))
        key = (tex, i % tex_pool)
        if key not in pool:
            pool[key] = value_noise_checker(tex, tex, seed + key[1], comps=4)
        frames.append(random_frame(rng, side, side, ntri, tex, seed + i, texture=pool[key]))
    return frames
