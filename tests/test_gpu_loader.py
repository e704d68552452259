"""A model loaded with Object.load_from_file (dg_obj_* + texture decoding)
renders on the GPU exactly as the CPU oracle renders the same parsed arrays,
under the reference's default scene (Scene::new: camera at (0, 0, 150) looking
at the origin, light at (0, 300, 300)), which frames models rescaled to |v| <= 100."""
import ctypes
import os

import numpy as np
import pytest

from draw_gb300 import imageio
from draw_gb300 import renderer as R
from draw_gb300 import scenes as S
from helpers import compare, describe, first_mismatch, oracle_render
from test_loader import _write_model

pytestmark = pytest.mark.gpu


def _desc_from_parse(lib, path, width=160, height=120):
    h = ctypes.c_void_p()
    assert lib.dg_obj_parse(os.fsencode(path), ctypes.byref(h)) == 0
    try:
        cnt = (ctypes.c_uint64 * 6)()
        lib.dg_obj_counts(h, cnt, 6)
        nv, nn, nuv, nmesh, nmat = (int(x) for x in cnt[:5])
        v, n, uv = np.zeros((nv, 3), np.float32), np.zeros((nn, 3), np.float32), np.zeros((nuv, 3), np.float32)
        lib.dg_obj_arrays(h, v.ctypes.data, n.ctypes.data, uv.ctypes.data)
        meshes = []
        for i in range(nmesh):
            nt, ti = ctypes.c_uint64(), ctypes.c_int32()
            lib.dg_obj_mesh(h, i, None, 0, ctypes.byref(nt), ctypes.byref(ti), None, 0)
            t = np.zeros((nt.value, 9), np.uint32)
            lib.dg_obj_mesh(h, i, t.ctypes.data, t.size, ctypes.byref(nt), ctypes.byref(ti), None, 0)
            meshes.append(S.MeshDesc(t, ti.value))
        textures, mats, paths = [], [], {}
        for i in range(nmat):
            m = R.dg_material()
            pa, pd = ctypes.create_string_buffer(1024), ctypes.create_string_buffer(1024)
            lib.dg_obj_material(h, i, ctypes.byref(m), None, 0, pa, pd, 1024)
            ids = []
            for p in (pa.value.decode(), pd.value.decode()):
                if p and p not in paths:
                    img, w, hh, c = imageio.read_image(p)
                    paths[p] = len(textures)
                    textures.append(S.TextureDesc(img, w, hh, c))
                ids.append(paths[p] if p else -1)
            mats.append(S.Material(tuple(m.ka), tuple(m.kd), tuple(m.ks), float(m.alpha), ids[0], ids[1]))
    finally:
        lib.dg_obj_free(h)
    return S.SceneDesc(width, height, textures=textures, objects=[S.ObjectDesc(v, n, uv, meshes, mats)])


def test_loaded_model_parity(gpu_ctx, oracle_lib, tmp_path):
    path = _write_model(tmp_path)
    desc = _desc_from_parse(gpu_ctx.lib, path)
    ref = oracle_render(desc)
    obj = R.Object.load_from_file(path, gpu_ctx)
    scene = R.Scene(desc.width, desc.height, gpu_ctx)  # Scene::new defaults
    scene.add_obj(obj)
    canvas = R.Canvas(desc.width, desc.height, gpu_ctx)
    canvas.init_depth(desc.clear_depth)
    scene.render(canvas)
    got = (*canvas.read(), 0)
    p = compare(ref, got, desc.clear_depth)
    print(describe(p))
    assert p.ok and p.n_covered > 200, f"{describe(p)}; {first_mismatch(ref, got)}"


@pytest.mark.parametrize("model", ["donut/donut.obj", "lemur/lemur.obj", "soldier1/soldier1.obj"])
def test_reference_model_parity(gpu_ctx, oracle_lib, model):
    """The reference's own models (vendored test data) loaded with
    Object.load_from_file and rendered at the reference's 800x600 window size
    under Scene::new's defaults: the donut has neither texture coordinates nor
    normals (the dummy-UV and generated smooth-normal paths, object.rs:368-429),
    the lemur carries a PNG diffuse map, soldier1 four materials without maps."""
    from test_loader import model_path

    path = model_path(model)
    if path is None:
        pytest.skip(f"{model} not present")
    desc = _desc_from_parse(gpu_ctx.lib, path, width=800, height=600)
    ref = oracle_render(desc)
    obj = R.Object.load_from_file(path, gpu_ctx)
    scene = R.Scene(desc.width, desc.height, gpu_ctx)
    scene.add_obj(obj)
    canvas = R.Canvas(desc.width, desc.height, gpu_ctx)
    canvas.init_depth(desc.clear_depth)
    for _ in range(2):  # a second frame into the same canvas renders the same
        scene.render(canvas)
        got = (*canvas.read(), 0)
        p = compare(ref, got, desc.clear_depth)
        assert p.ok and p.n_covered > 1000, f"{model}: {describe(p)}; {first_mismatch(ref, got)}"
