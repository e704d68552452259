"""A second, independent restatement of the reference render path in pure
Python with numpy float32 scalars (test infrastructure, tiny scenes only).

It is written separately from oracle/draw_oracle.cpp and is used to
cross-check that oracle on small seeded scenes. It follows the reference
renderer (mororo18/draw, Rust): src/renderer/linalg.rs, canvas.rs:577-960,
scene/mod.rs:12-100, 154-168, 296-747, 817-1088. The opaque pass only.
"""
from __future__ import annotations

import math

import numpy as np

F = np.float32
INF = F(np.inf)


def f(x) -> np.float32:
    return F(x)


# ---- linalg.rs ---------------------------------------------------------
def v_add(a, b):
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def v_sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def v_scale(a, s):
    return (a[0] * s, a[1] * s, a[2] * s)


def v_div(a, s):
    return (a[0] / s, a[1] / s, a[2] / s)


def v_dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def v_norm(a):
    return np.sqrt((a[0] * a[0] + a[1] * a[1]) + a[2] * a[2])


def v_unit(a):
    return v_div(a, v_norm(a))


def v_cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def m_mul(A, B):
    C = [[F(0)] * 4 for _ in range(4)]
    for i in range(4):
        for j in range(4):
            acc = F(0)
            for k in range(4):
                acc = acc + A[i][k] * B[k][j]
            C[i][j] = acc
    return C


def m_vec(A, v):
    out = []
    for i in range(4):
        acc = F(0)
        for j in range(4):
            acc = acc + A[i][j] * v[j]
        out.append(acc)
    return out


def usize(x) -> int:
    """Rust `as usize` from f32."""
    if not (x > 0):
        return 0
    if x >= F(2.0 ** 64):
        return 2 ** 64 - 1
    return int(x)


def u8(x) -> int:
    if not (x > 0):
        return 0
    if x >= F(255):
        return 255
    return int(x)


# ---- camera, scene/mod.rs:296-594, 817-899 -----------------------------
def camera(pos, direction, ratio, near, far, fov_x):
    pos = tuple(f(x) for x in pos)
    direction = tuple(f(x) for x in direction)
    rad = f(fov_x) * (f(math.pi) / f(180.0))
    half = rad / f(2.0)
    right = abs(f(near)) * f(math.tan(float(half)))
    top = (f(1.0) / f(ratio)) * right
    return dict(pos=pos, dir=v_unit(direction), right=right, left=-right, top=top, bottom=-top, near=f(near),
                far=f(far))


def basis(cam):
    up = (f(0), f(1), f(0))
    g = cam["dir"]
    w = v_scale(v_div(g, v_norm(g)), f(-1.0))
    txw = v_cross(up, w)
    u = v_div(txw, v_norm(txw))
    v = v_cross(w, u)
    u, v, w = v_unit(u), v_unit(v), v_unit(w)
    z = F(0)
    return [[u[0], v[0], w[0], z], [u[1], v[1], w[1], z], [u[2], v[2], w[2], z], [z, z, z, F(1)]]


def transform(cam, width, height):
    B = basis(cam)
    Bt = [[B[j][i] for j in range(4)] for i in range(4)]
    p = cam["pos"]
    z, o = F(0), F(1)
    T = [[o, z, z, -p[0]], [z, o, z, -p[1]], [z, z, o, -p[2]], [z, z, z, o]]
    view = m_mul(Bt, T)
    n, fa, r, l, t, b = cam["near"], cam["far"], cam["right"], cam["left"], cam["top"], cam["bottom"]
    persp = [[n, z, z, z], [z, n, z, z], [z, z, n + fa, -(n * fa)], [z, z, o, z]]
    orth = [[F(2) / (r - l), z, z, -(r + l) / (r - l)], [z, F(2) / (t - b), z, -(t + b) / (t - b)],
            [z, z, F(2) / (n - fa), -(n + fa) / (n - fa)], [z, z, z, o]]
    nx, ny = F(width), F(height)
    vp = [[nx / F(2), z, z, (nx - o) / F(2)], [z, ny / F(2), z, (ny - o) / F(2)], [z, z, o, z], [z, z, z, o]]
    return m_mul(m_mul(m_mul(vp, orth), persp), view)


def planes(cam):
    B = basis(cam)
    p = cam["pos"]
    n, fa, r, l, t, b = cam["near"], cam["far"], cam["right"], cam["left"], cam["top"], cam["bottom"]

    def world(x, y, zz):
        h = m_vec(B, [x, y, zz, F(1)])
        return v_add((h[0] / h[3], h[1] / h[3], h[2] / h[3]), p)

    urn, uln, lrn, lln = world(r, t, n), world(l, t, n), world(r, b, n), world(l, b, n)
    xc, yc = (l + r) / F(2), (b + t) / F(2)
    ucf, lcf = world(xc, (fa * t) / n, fa), world(xc, (fa * b) / n, fa)
    rcf, lfc = world((fa * r) / n, yc, fa), world((fa * l) / n, yc, fa)
    vis = v_div(v_add(urn, lcf), F(2))
    out = []
    for a, bb, c in [(urn, lrn, lln), (lfc, rcf, ucf), (rcf, urn, lrn), (lfc, lln, uln), (ucf, uln, urn),
                     (lcf, lln, lrn)]:
        pv, qv = v_sub(bb, a), v_sub(c, bb)
        nn = v_cross(pv, qv)
        k = -v_dot(nn, a)
        if v_dot(nn, vis) + k < 0:
            nn = v_cross(qv, pv)
            k = -v_dot(nn, a)
            assert v_dot(nn, vis) + k > 0
        out.append((nn, k))
    return out


def plane_f(pl, pt):
    return v_dot(pl[0], pt) + pl[1]


# ---- clipping, scene/mod.rs:43-90, 641-746 ------------------------------
def lerp_attr(a, c, t):
    """a + (c - a) * t for every field of a vertex record (dict of tuples/scalars)."""
    out = {}
    for key in a:
        if isinstance(a[key], tuple):
            out[key] = tuple(x + (y - x) * t for x, y in zip(a[key], c[key]))
        else:
            out[key] = a[key] + (c[key] - a[key]) * t
    return out


def clip_plane(pl, tri):
    (a, aa), (b, ba), (c, ca) = tri
    fa, fb, fc = plane_f(pl, a), plane_f(pl, b), plane_f(pl, c)
    if fa > 0 and fb > 0 and fc > 0:
        return [tri]
    if fa <= 0 and fb <= 0 and fc <= 0:
        return []
    if fa * fc >= 0:
        (a, aa, fa), (b, ba, fb), (c, ca, fc) = (c, ca, fc), (a, aa, fa), (b, ba, fb)
    elif fb * fc >= 0:
        (a, aa, fa), (b, ba, fb), (c, ca, fc) = (b, ba, fb), (c, ca, fc), (a, aa, fa)
    eps = F(0.0000001)
    ta = plane_f(pl, a) / v_dot(pl[0], v_sub(a, c)) - eps
    na = v_add(a, v_scale(v_sub(c, a), ta))
    naa = lerp_attr(aa, ca, ta)
    tb = plane_f(pl, b) / v_dot(pl[0], v_sub(b, c)) - eps
    nb = v_add(b, v_scale(v_sub(c, b), tb))
    nba = lerp_attr(ba, ca, tb)
    if fc <= 0:
        return [((a, aa), (na, naa), (nb, nba)), ((a, aa), (b, ba), (nb, nba))]
    return [((c, ca), (na, naa), (nb, nba))]


def clip(pls, tri):
    for p in pls[2:6]:
        fs = [plane_f(p, v[0]) for v in tri]
        if all(x <= 0 for x in fs):
            return []
    pool = [tri]
    for p in pls[0:2]:
        pool = [o for t in pool for o in clip_plane(p, t)]
    return pool


# ---- raster + shading, canvas.rs:577-750, 896-930 -----------------------
def edge(p, q, x, y):
    return (p[1] - q[1]) * x + (q[0] - p[0]) * y + p[0] * q[1] - q[0] * p[1]


def axis_range(vals, size):
    mn, mx = INF, -INF
    for v in vals:
        if v < mn:
            mn = v
    for v in vals:
        if v > mx:
            mx = v
    lo0, hi0 = usize(mn), usize(mx)
    lo, hi = min(lo0, hi0), max(lo0, hi0)
    hi = min(hi, size - 1)
    if lo > hi:
        lo, hi = 0, 0
    return lo, hi


def texel(img, w, h, comps, u, v):
    ui = usize(np.floor(u * (F(w) - F(1))))
    vi = (h - 1 - usize(np.floor(v * (F(h) - F(1))))) % 2 ** 64
    off = ((vi * w + ui) * comps) % 2 ** 64
    if off + 3 > len(img):
        raise IndexError("texel offset out of range")
    return [F(int(img[off + k])) / F(255) for k in range(3)]


def texel_bilinear(img, w, h, comps, u, v):
    """Extension (no counterpart in the reference): the bilinear blend of the
    base texel (addressed like the nearest one) and its right, upper and
    upper-right neighbours (clamped at the image's last column and first row),
    per channel t0 = c00 (1 - ax) + c01 ax, t1 = c10 (1 - ax) + c11 ax,
    c = t0 (1 - ay) + t1 ay."""
    x, y = u * (F(w) - F(1)), v * (F(h) - F(1))
    fx, fy = np.floor(x), np.floor(y)
    ax, ay = x - fx, y - fy
    ui = usize(fx)
    vi = (h - 1 - usize(fy)) % 2 ** 64
    o00 = ((vi * w + ui) * comps) % 2 ** 64
    dx = comps if ui + 1 < w else 0
    dy = w * comps if 1 <= vi < h else 0
    offs = [o00, (o00 + dx) % 2 ** 64, (o00 - dy) % 2 ** 64, (o00 - dy + dx) % 2 ** 64]
    for o in offs:
        if o + 3 > len(img):
            raise IndexError("texel offset out of range")
    out = []
    for k in range(3):
        c00, c01, c10, c11 = (F(int(img[o + k])) / F(255) for o in offs)
        t0 = c00 * (F(1) - ax) + c01 * ax
        t1 = c10 * (F(1) - ax) + c11 * ax
        out.append(t0 * (F(1) - ay) + t1 * ay)
    return out


def sample(img, w, h, comps, filt, u, v):
    return texel_bilinear(img, w, h, comps, u, v) if filt else texel(img, w, h, comps, u, v)


def powi(x, e):
    r = F(1)
    n = e
    while True:
        if n & 1:
            r = r * x
        n >>= 1
        if n == 0:
            break
        x = x * x
    return r


def render(desc):
    """Returns (bgra (H,W,4) uint8, depth (H,W) float32) for a SceneDesc (opaque meshes only)."""
    W, H = desc.canvas_size
    frame = np.zeros((H, W, 4), np.uint8)
    frame[...] = (255, 186, 155, 255)
    depth = np.full((H, W), F(desc.clear_depth), np.float32)
    with np.errstate(all="ignore"):
        cam = camera(desc.cam_pos, desc.cam_dir, desc.ratio, desc.near, desc.far, desc.fov_x)
        M = transform(cam, desc.width, desc.height)
        pls = planes(cam)
        cp = cam["pos"]
        lights = [tuple(f(x) for x in l) for l in desc.lights]
        off = (F(desc.offset[0]), F(desc.offset[1]))
        for ob in desc.objects:
            V = [tuple(f(x) for x in p) for p in ob.vertices]
            visual = []
            for p in V:
                ed = v_sub(p, cp)
                eye = v_unit(ed)
                ls = [v_unit(v_sub(p, L)) for L in lights]
                visual.append(dict(depth=v_norm(ed), light=ls, half=[v_unit(v_add(l, eye)) for l in ls]))
            for mesh in ob.meshes:
                mat = ob.materials[mesh.texture_idx]
                if not (mat.alpha >= 1.0) and not np.isnan(mat.alpha):
                    continue
                maps = []
                for mi in (mat.map_kd, mat.map_ka):
                    if mi < 0:
                        maps.append((np.array([255, 255, 255], np.uint8), 1, 1, 3, 0))
                    else:
                        t = desc.textures[mi]
                        maps.append((t.img, t.width, t.height, t.comps, getattr(t, "filter", 0)))
                for row in mesh.tris:
                    vi, ti, ni = row[0:3], row[3:6], row[6:9]
                    a, b, c = V[vi[0]], V[vi[1]], V[vi[2]]
                    n = v_cross(v_sub(b, a), v_sub(c, b))
                    ctr = v_div(v_add(v_add(v_add((F(0), F(0), F(0)), a), b), c), F(3))
                    if v_dot(v_sub(cp, ctr), n) <= 0:
                        continue
                    verts = []
                    for k in range(3):
                        vis = visual[vi[k]]
                        attr = dict(depth=vis["depth"], normal=tuple(f(x) for x in ob.normals[ni[k]]),
                                    uv=tuple(f(x) for x in ob.uvs[ti[k]]))
                        for li in range(len(lights)):
                            attr[f"l{li}"] = vis["light"][li]
                            attr[f"h{li}"] = vis["half"][li]
                        verts.append((V[vi[k]], attr))
                    for tri in clip(pls, tuple(verts)):
                        centres, ws = [], []
                        for p, _ in tri:
                            hh = m_vec(M, [p[0], p[1], p[2], F(1)])
                            sx, sy = hh[0] / hh[3], hh[1] / hh[3]
                            ws.append(hh[3])
                            centres.append((np.floor((sx + (-off[0])) + F(0.5)), np.floor((sy + (-off[1])) + F(0.5))))
                        _raster(tri, centres, mat, maps, len(lights), desc.exponent, W, H, frame, depth, ws,
                                getattr(desc, "interpolation", 0))
    return frame, depth


def _raster(tri, cs, mat, maps, nl, exponent, W, H, frame, depth, ws, interp):
    A, B, C = cs
    x0, x1 = axis_range([A[0], B[0], C[0]], W)
    y0, y1 = axis_range([A[1], B[1], C[1]], H)
    fa, fb, fg = edge(B, C, A[0], A[1]), edge(C, A, B[0], B[1]), edge(A, B, C[0], C[1])
    ta = fa * edge(B, C, F(-1), F(-1)) > 0
    tb = fb * edge(C, A, F(-1), F(-1)) > 0
    tg = fg * edge(A, B, F(-1), F(-1)) > 0
    at = [v[1] for v in tri]
    ks, kd, ka = [tuple(f(x) for x in m) for m in (mat.ks, mat.kd, mat.ka)]
    for y in range(y0, y1 + 1):
        for x in range(x0, x1 + 1):
            xf, yf = F(x), F(y)
            al = edge(B, C, xf, yf) / fa
            be = edge(C, A, xf, yf) / fb
            ga = edge(A, B, xf, yf) / fg
            if not (al >= 0 and be >= 0 and ga >= 0):
                continue
            if not ((al > 0 or ta) and (be > 0 or tb) and (ga > 0 or tg)):
                continue

            def mix(key, wa, wb, wc):
                u, v, w = at[0][key], at[1][key], at[2][key]
                if isinstance(u, tuple):
                    return tuple((p * wa + q * wb) + r * wc for p, q, r in zip(u, v, w))
                return (wa * u + wb * v) + wc * w

            d = mix("depth", al, be, ga)
            if interp:  # extension: attributes weighted by 1/w, depth and coverage as the reference
                pa, pb, pc = al * (F(1) / ws[0]), be * (F(1) / ws[1]), ga * (F(1) / ws[2])
                s = (pa + pb) + pc
                al, be, ga = pa / s, pb / s, pc / s
            uv = mix("uv", al, be, ga)
            dif = sample(*maps[0], uv[0], uv[1])
            amb = sample(*maps[1], uv[0], uv[1])
            nrm = mix("normal", al, be, ga)
            c_r = tuple(dif[i] * kd[i] for i in range(3))
            c_a = tuple(amb[i] * ka[i] for i in range(3))
            inner = c_a
            for li in range(nl):
                ln = v_dot(mix(f"l{li}", al, be, ga), nrm)
                mx = ln if ln > 0 else F(0)
                inner = v_add(inner, v_scale(ks, F(1) - mx))
            col = tuple(c_r[i] * inner[i] for i in range(3))
            for li in range(nl):
                col = v_add(col, v_scale(ks, powi(v_dot(mix(f"h{li}", al, be, ga), nrm), exponent)))
            sc = v_scale(col, F(255))
            if d < depth[y, x]:
                frame[H - 1 - y, x] = (u8(sc[2]), u8(sc[1]), u8(sc[0]), 255)
                depth[y, x] = d
