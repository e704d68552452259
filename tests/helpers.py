"""Shared test helpers: render one SceneDesc with the CPU oracle and with the GPU
library, and compare the two frames with the parity bar (coverage and depth
bit-exact, colour within 1 LSB per channel)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# Colour tolerance of the parity bar: at most 1 LSB per channel.
COLOUR_TOL_LSB = 1


def oracle_render(desc, o=None, frames: int = 1, camera_ops=()):
    """Renders desc with the oracle; returns (bgra, depth, status)."""
    import oracle as _oracle

    o = o or _oracle.Oracle()
    texs = [o.texmap(t.img, t.width, t.height, t.comps) for t in desc.textures]
    for t, i in zip(desc.textures, texs):
        if getattr(t, "filter", 0):
            o.set_filter(i, t.filter)
    s = o.scene(desc.width, desc.height)
    o.set_camera(s, desc.cam_pos, desc.cam_dir, desc.ratio, desc.near, desc.far, desc.fov_x)
    o.set_lights(s, desc.lights)
    o.set_exponent(s, desc.exponent)
    if getattr(desc, "interpolation", 0):
        o.set_interpolation(s, desc.interpolation)
    for ob in desc.objects:
        mats = [dict(ka=m.ka, kd=m.kd, ks=m.ks, alpha=m.alpha, map_ka=texs[m.map_ka] if m.map_ka >= 0 else -1,
                     map_kd=texs[m.map_kd] if m.map_kd >= 0 else -1) for m in ob.materials]
        oid = o.object(ob.vertices, ob.normals, ob.uvs, [(m.tris, m.texture_idx) for m in ob.meshes], mats)
        o.add_obj(s, oid)
    cw, ch = desc.canvas_size
    c = o.canvas(cw, ch)
    o.init_depth(c, desc.clear_depth)
    o.apply_offset(c, *desc.offset)
    st = 0
    for _ in range(frames):
        for op, args in camera_ops:
            o.camera_op(s, op, args)
        st = o.render(s, c)
        if st:
            break
    f = o.read(c, cw, ch)
    return f.bgra, f.depth, st


def oracle_render_many(descs, threads: int | None = None):
    """oracle_render of every desc, on host threads (one oracle context per
    call; ctypes releases the GIL while a frame renders)."""
    import concurrent.futures as cf
    import os

    n = threads or min(len(descs), os.cpu_count() or 1) or 1
    with cf.ThreadPoolExecutor(n) as ex:
        return list(ex.map(oracle_render, descs))


def gpu_render(desc, ctx, frames: int = 1, camera_ops=()):
    """Renders desc through the C ABI; returns (bgra, depth, status)."""
    from draw_gb300 import renderer

    b = renderer.build_scene(desc, ctx)
    st = 0
    try:
        for _ in range(frames):
            for op, args in camera_ops:
                b.scene.camera._op(op, *args)
            b.scene.render(b.canvas)
        bgra, depth = b.canvas.read()
    except renderer.DrawError as e:
        st = e.status
        bgra, depth = None, None
    return bgra, depth, st


@dataclass
class Parity:
    coverage_equal: bool
    depth_bits_equal: bool
    colour_max_lsb: int
    colour_frac_diff: float
    n_covered: int

    @property
    def ok(self) -> bool:
        return self.coverage_equal and self.depth_bits_equal and self.colour_max_lsb <= COLOUR_TOL_LSB


def compare(ref, got, clear_depth=float("inf")) -> Parity:
    rb, rd = ref[0], ref[1]
    gb, gd = got[0], got[1]
    rcov = rd.view(np.uint32) != np.float32(clear_depth).view(np.uint32)
    gcov = gd.view(np.uint32) != np.float32(clear_depth).view(np.uint32)
    diff = np.abs(rb.astype(np.int16) - gb.astype(np.int16))
    px = diff.max(axis=-1) if diff.size else diff
    return Parity(
        coverage_equal=bool(np.array_equal(rcov, gcov)),
        depth_bits_equal=bool(np.array_equal(rd.view(np.uint32), gd.view(np.uint32))),
        colour_max_lsb=int(diff.max()) if diff.size else 0,
        colour_frac_diff=float((px > 0).mean()) if diff.size else 0.0,
        n_covered=int(rcov.sum()),
    )


def describe(p: Parity) -> str:
    return (f"coverage_equal={p.coverage_equal} depth_bits_equal={p.depth_bits_equal} "
            f"colour_max_lsb={p.colour_max_lsb} colour_frac_diff={p.colour_frac_diff:.3g} covered={p.n_covered}")


def first_mismatch(ref, got):
    rd, gd = ref[1].view(np.uint32), got[1].view(np.uint32)
    idx = np.argwhere(rd != gd)
    if len(idx):
        y, x = idx[0]
        return f"depth mismatch at y={y} x={x}: ref={ref[1][y, x]!r} got={got[1][y, x]!r} (count {len(idx)})"
    d = np.argwhere(np.abs(ref[0].astype(int) - got[0].astype(int)).max(-1) > COLOUR_TOL_LSB)
    if len(d):
        y, x = d[0]
        return f"colour mismatch at row={y} x={x}: ref={ref[0][y, x]} got={got[0][y, x]} (count {len(d)})"
    return "none"
