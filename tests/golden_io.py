"""Serialization of a SceneDesc and its rendered frame into one .npz fixture, so
golden tests do not depend on how a platform rounds the generators' float64
trigonometry."""
from __future__ import annotations

import numpy as np

from draw_gb300 import scenes as S


def save(path, desc, bgra, depth, status=0):
    d = {
        "width": desc.width, "height": desc.height, "cam_pos": np.array(desc.cam_pos, np.float32),
        "cam_dir": np.array(desc.cam_dir, np.float32), "near": desc.near, "far": desc.far, "fov_x": desc.fov_x,
        "lights": np.asarray(desc.lights, np.float32), "exponent": desc.exponent, "clear_depth": desc.clear_depth,
        "offset": np.array(desc.offset, np.int32),
        "canvas_wh": np.array(desc.canvas_size, np.int64), "n_tex": len(desc.textures),
        "n_obj": len(desc.objects), "bgra": bgra, "depth": depth, "status": status,
        "interpolation": int(getattr(desc, "interpolation", 0)),
    }
    for i, t in enumerate(desc.textures):
        d[f"tex{i}_img"] = t.img
        d[f"tex{i}_shape"] = np.array([t.width, t.height, t.comps], np.int64)
        d[f"tex{i}_filter"] = int(getattr(t, "filter", 0))
    for i, o in enumerate(desc.objects):
        d[f"obj{i}_v"] = o.vertices
        d[f"obj{i}_n"] = o.normals
        d[f"obj{i}_uv"] = o.uvs
        d[f"obj{i}_nmesh"] = len(o.meshes)
        for j, m in enumerate(o.meshes):
            d[f"obj{i}_mesh{j}_tris"] = m.tris
            d[f"obj{i}_mesh{j}_tex"] = m.texture_idx
        d[f"obj{i}_mats"] = np.array([[*m.ka, *m.kd, *m.ks, m.alpha, m.map_ka, m.map_kd] for m in o.materials],
                                     np.float64)
    np.savez_compressed(path, **d)


def load(path):
    z = np.load(path)
    textures = []
    for i in range(int(z["n_tex"])):
        w, h, c = (int(x) for x in z[f"tex{i}_shape"])
        t = S.TextureDesc(z[f"tex{i}_img"], w, h, c)
        if f"tex{i}_filter" in z.files:  # the opt-in bilinear filter (older fixtures: nearest)
            t.filter = int(z[f"tex{i}_filter"])
        textures.append(t)
    objects = []
    for i in range(int(z["n_obj"])):
        meshes = [S.MeshDesc(z[f"obj{i}_mesh{j}_tris"], int(z[f"obj{i}_mesh{j}_tex"]))
                  for j in range(int(z[f"obj{i}_nmesh"]))]
        mats = [S.Material(tuple(r[0:3]), tuple(r[3:6]), tuple(r[6:9]), float(r[9]), int(r[10]), int(r[11]))
                for r in z[f"obj{i}_mats"]]
        objects.append(S.ObjectDesc(z[f"obj{i}_v"], z[f"obj{i}_n"], z[f"obj{i}_uv"], meshes, mats))
    cw, ch = (int(x) for x in z["canvas_wh"])
    desc = S.SceneDesc(int(z["width"]), int(z["height"]), cam_pos=tuple(float(x) for x in z["cam_pos"]),
                       cam_dir=tuple(float(x) for x in z["cam_dir"]), near=float(z["near"]), far=float(z["far"]),
                       fov_x=float(z["fov_x"]), lights=z["lights"], exponent=int(z["exponent"]),
                       clear_depth=float(z["clear_depth"]), offset=tuple(int(x) for x in z["offset"]),
                       canvas_wh=(cw, ch), textures=textures, objects=objects)
    if "interpolation" in z.files:  # the opt-in perspective-correct mode (older fixtures: screen space)
        desc.interpolation = int(z["interpolation"])
    return desc, z["bgra"], z["depth"], int(z["status"])
