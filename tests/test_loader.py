"""The OBJ/MTL loader (dg_obj_*, restating Object::load_from_file,
object.rs:106-454) and the PNG/PPM texture decoder (in place of stb_image).

The parser is checked bit for bit against an independent restatement in
numpy float32 below (the same rules: quad split (a,b,c),(c,d,a); normals
normalized; positions scaled to max |v| = 100; per-group dummy texture
coordinate and generated smooth normals; materials after Texture::default()).
The reference's own model files are parsed too (triangle counts): the donut,
lemur and soldier1 models are vendored under tests/fixtures/models as test
data; fgc_skeleton (whose material lacks Ka, on which the reference panics) is
parsed when DRAW_REF_MODELS names a directory holding the reference's models."""
import ctypes
import os
import struct
import zlib

import numpy as np
import pytest

from draw_gb300 import imageio
from draw_gb300 import renderer as R

F = np.float32
FIXTURE_MODELS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fixtures", "models")
REF_MODELS = os.environ.get("DRAW_REF_MODELS", "")


def model_path(model: str) -> str | None:
    """A model file from the vendored fixtures, else from DRAW_REF_MODELS."""
    for root in (FIXTURE_MODELS, REF_MODELS):
        if root and os.path.exists(os.path.join(root, model)):
            return os.path.join(root, model)
    return None


OBJ_TEXT = """# quads, triangles, groups, materials, negative indices
mtllib m.mtl
v 1 0 0
v 2 0.5 -1
v 0 3 0.25
v -1.5 -0.5 2
v 0.5 -2 1
v 4 1 1
vt 0 0
vt 1 0
vt 1 1
vt 0.25 0.75
vn 0 0 2
vn 1 1 0
vn 0 -3 4
o first
g shell
usemtl red
f 1/1/1 2/2/2 3/3/3 4/4/1
f 2/2/2 5/3/3 6/4/1
usemtl glass
f -1/-1/-1 -2/-2/-2 -3/-3/-3
g bare
f 1 3 5
f 2 4 6 1
g mixed
usemtl missing_name
f 1//1 2//2 3//3
f 4/1 5/2 6/3
f 3 4 5
"""

MTL_TEXT = """newmtl red
Ka 0.1 0.0 0.0
Kd 0.8 0.1 0.1
Ks 0.5 0.5 0.5
newmtl glass
Ka 0 0 0
Kd 0.2 0.3 0.9
Ks 1 1 1
d 0.4
map_Kd glass.png
"""


def _restate(pos, uvs, nrm, groups, materials):
    """The loader's rules in numpy float32 (an independent restatement)."""
    pos = np.array(pos, F)
    nrm = [np.array(n, F) for n in nrm]
    nrm = [n / np.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2], dtype=F) for n in nrm]
    uv = [np.array([u[0], u[1], 0.0], F) for u in uvs]
    norms = np.array([np.sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2], dtype=F) for p in pos], F)
    factor = F(100.0) / norms.max()
    pos = pos * factor
    names = ["default"] + [m for m in materials]
    meshes = []
    for gname, mat, faces in groups:
        tris, miss_t, miss_n = [], False, False
        for face in faces:
            ft = any(c[1] is None for c in face)
            fn = any(c[2] is None for c in face)
            miss_t |= ft
            miss_n |= fn
            for order in ([0, 1, 2], [2, 3, 0])[:(2 if len(face) == 4 else 1)]:
                tris.append(([face[k][0] for k in order], None if ft else [face[k][1] for k in order],
                             None if fn else [face[k][2] for k in order]))
        if miss_t:
            d = len(uv)
            uv.append(np.zeros(3, F))
            tris = [(a, b if b is not None else [d] * 3, c) for a, b, c in tris]
        if miss_n:
            gen = [np.zeros(3, F) for _ in range(len(pos))]
            for a, _, _ in tris:
                A, B, C = pos[a[0]], pos[a[1]], pos[a[2]]
                p, q = B - A, C - B
                n = np.array([p[1] * q[2] - p[2] * q[1], p[2] * q[0] - p[0] * q[2], p[0] * q[1] - p[1] * q[0]], F)
                for k in range(3):
                    gen[a[k]] = gen[a[k]] + n
            base = len(nrm)
            tris = [(a, b, c if c is not None else [x + base for x in a]) for a, b, c in tris]
            with np.errstate(invalid="ignore"):
                nrm += [g / np.sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2], dtype=F) for g in gen]
        tidx = names.index(mat) if mat in names else 0
        meshes.append((gname, np.array([a + b + c for a, b, c in tris], np.uint32), tidx))
    return pos, np.array(nrm, F), np.array(uv, F), meshes


def _parse(lib, path):
    h = ctypes.c_void_p()
    st = lib.dg_obj_parse(os.fsencode(path), ctypes.byref(h))
    return st, h


@pytest.fixture(scope="module")
def lib():
    from draw_gb300 import _build

    _build.build()
    return R.load_library()


def _write_png(path, img, filt):
    """Test-local PNG encoder using one filter type for every row."""
    h, w, c = img.shape
    stride = w * c
    a = img.reshape(h, stride).astype(np.int32)
    rows = []
    for y in range(h):
        cur, prev = a[y], a[y - 1] if y else np.zeros(stride, np.int32)
        left = np.concatenate([np.zeros(c, np.int32), cur[:-c]])
        ul = np.concatenate([np.zeros(c, np.int32), prev[:-c]])
        if filt == 0:
            out = cur
        elif filt == 1:
            out = cur - left
        elif filt == 2:
            out = cur - prev
        elif filt == 3:
            out = cur - ((left + prev) >> 1)
        else:
            p = left + prev - ul
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - ul)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, ul))
            out = cur - pred
        rows.append(bytes([filt]) + (out & 0xFF).astype(np.uint8).tobytes())

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, {3: 2, 4: 6}[c], 0, 0, 0)) +
                chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b""))


@pytest.mark.parametrize("filt", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("comps", [3, 4])
def test_png_filters_round_trip(tmp_path, filt, comps):
    rng = np.random.default_rng(filt * 10 + comps)
    img = rng.integers(0, 256, (13, 17, comps), dtype=np.uint8)
    p = str(tmp_path / "t.png")
    _write_png(p, img, filt)
    got, w, h, c = imageio.read_png(p)
    assert (w, h, c) == (17, 13, comps) and np.array_equal(got.reshape(13, 17, comps), img)


def _write_model(d):
    (d / "m.obj").write_text(OBJ_TEXT)
    (d / "m.mtl").write_text(MTL_TEXT)
    img = np.zeros((4, 6, 4), np.uint8)
    img[..., 0] = np.arange(6)[None] * 40
    img[..., 3] = 255
    _write_png(str(d / "glass.png"), img, 4)
    return str(d / "m.obj")


def test_parser_matches_restatement(lib, tmp_path):
    path = _write_model(tmp_path)
    st, h = _parse(lib, path)
    assert st == 0
    try:
        cnt = (ctypes.c_uint64 * 6)()
        assert lib.dg_obj_counts(h, cnt, 6) == 0
        nv, nn, nuv, nmesh, nmat, ntri = list(cnt)
        v, n, uv = np.zeros((nv, 3), F), np.zeros((nn, 3), F), np.zeros((nuv, 3), F)
        assert lib.dg_obj_arrays(h, v.ctypes.data, n.ctypes.data, uv.ctypes.data) == 0
        P = [[1, 0, 0], [2, 0.5, -1], [0, 3, 0.25], [-1.5, -0.5, 2], [0.5, -2, 1], [4, 1, 1]]
        T = [[0, 0], [1, 0], [1, 1], [0.25, 0.75]]
        N = [[0, 0, 2], [1, 1, 0], [0, -3, 4]]
        c = lambda s: tuple(None if x == "" else int(x) - 1 for x in (s.split("/") + ["", ""])[:3])  # noqa: E731
        groups = [("shell", "red", [[c("1/1/1"), c("2/2/2"), c("3/3/3"), c("4/4/1")], [c("2/2/2"), c("5/3/3"), c("6/4/1")]]),
                  ("shell", "glass", [[(5, 3, 2), (4, 2, 1), (3, 1, 0)]]),
                  ("bare", "glass", [[c("1"), c("3"), c("5")], [c("2"), c("4"), c("6"), c("1")]]),
                  ("mixed", "missing_name", [[c("1//1"), c("2//2"), c("3//3")], [c("4/1"), c("5/2"), c("6/3")],
                                             [c("3"), c("4"), c("5")]])]
        rp, rn, ruv, rmeshes = _restate(P, T, N, groups, ["red", "glass"])
        assert np.array_equal(v.view(np.uint32), rp.view(np.uint32))
        assert np.array_equal(uv, ruv)
        assert n.shape == rn.shape and np.array_equal(n.view(np.uint32), rn.view(np.uint32))
        assert nmesh == len(rmeshes) and nmat == 3 and ntri == sum(len(m[1]) for m in rmeshes)
        name = ctypes.create_string_buffer(256)
        for i, (gname, tris, tidx) in enumerate(rmeshes):
            nt, ti = ctypes.c_uint64(), ctypes.c_int32()
            t = np.zeros((len(tris), 9), np.uint32)
            assert lib.dg_obj_mesh(h, i, t.ctypes.data, t.size, ctypes.byref(nt), ctypes.byref(ti), name, 256) == 0
            assert name.value.decode() == gname and ti.value == tidx and np.array_equal(t, tris), i
        m = R.dg_material()
        pa, pd = ctypes.create_string_buffer(512), ctypes.create_string_buffer(512)
        assert lib.dg_obj_material(h, 2, ctypes.byref(m), name, 256, pa, pd, 512) == 0
        assert name.value == b"glass" and abs(m.alpha - 0.4) < 1e-7 and pa.value == b""
        assert pd.value.decode() == str(tmp_path / "glass.png")
        assert lib.dg_obj_material(h, 0, ctypes.byref(m), name, 256, pa, pd, 512) == 0  # Texture::default()
        assert name.value == b"default" and list(m.ka) == [F(0.9)] * 3 and list(m.kd) == [F(0.4)] * 3
    finally:
        lib.dg_obj_free(h)


@pytest.mark.parametrize("text,status", [
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nv 2 2 2\nf 1 2 3 4 5\n", 8),  # more than 4 vertices: todo!()
    ("v 0 0 0\nv 1 0 0\nf 1 2\n", 1),                                   # vertex_index[2] out of bounds
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 7\n", 2),                        # index past the positions
    ("mtllib none.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", 1),       # library that does not open
    ("f 1 2 3\n", 1),                                                   # no positions
])
def test_parser_errors(lib, tmp_path, text, status):
    p = tmp_path / "bad.obj"
    p.write_text(text)
    st, h = _parse(lib, str(p))
    if st == 0:
        lib.dg_obj_free(h)
    assert st == status
    assert _parse(lib, str(tmp_path / "missing.obj"))[0] == 1


def test_load_from_file_python_mirror(lib, tmp_path):
    """Object.load_from_file over a host-only context: textures decoded, meshes and materials passed on."""
    path = _write_model(tmp_path)
    st, h = _parse(lib, path)
    assert st == 0
    lib.dg_obj_free(h)
    img, w, hh, comps = imageio.read_image(str(tmp_path / "glass.png"))
    assert (w, hh, comps) == (6, 4, 4)


@pytest.mark.parametrize("model,ntri,status", [("donut/donut.obj", 2048, 0), ("lemur/lemur.obj", 1972, 0),
                                               ("soldier1/soldier1.obj", 3144, 0),
                                               ("skeleton/fgc_skeleton.obj", 0, 1)])
def test_reference_models(lib, model, ntri, status):
    path = model_path(model)
    if path is None:
        pytest.skip(f"{model} is not vendored and DRAW_REF_MODELS is not set")
    st, h = _parse(lib, path)
    assert st == status
    if st == 0:
        cnt = (ctypes.c_uint64 * 6)()
        lib.dg_obj_counts(h, cnt, 6)
        lib.dg_obj_free(h)
        assert cnt[5] == ntri
