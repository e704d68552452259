"""Regenerates the golden fixtures in tests/golden/ with the CPU oracle.

Each fixture holds a small seeded scene (inputs included) and the frame the
oracle renders for it. The reference renderer itself cannot be run here (Rust,
no toolchain), so these pin the oracle against regressions and pin the GPU path
to fixed bytes; the oracle is cross-checked separately against an independent
Python restatement and hand-derived known answers.

Usage: python tests/golden/make_golden.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import cases  # noqa: E402
import golden_io  # noqa: E402
from draw_gb300 import scenes as S  # noqa: E402
from helpers import oracle_render  # noqa: E402


def golden_cases():
    out = {
        "tie_rule": cases.tie_rule_scene(),
        "equal_depth": cases.equal_depth_scene(),
        "clip": cases.clip_scene(),
        "degenerate": cases.degenerate_scene(),
        "multi_object": cases.multi_object_scene(),
        "reference_default": cases.reference_default_scene(160, 120),
        "torus_small": S.torus_scene(width=160, height=120, nu=24, nv=10, tex=64),
        "texture_range": cases.texture_range_scene(),
    }
    off = S.torus_scene(width=200, height=140, nu=20, nv=10, tex=32, exponent=2)
    off.offset, off.canvas_wh, off.clear_depth = (60, 40), (80, 60), 100000.0
    out["offset_collapse"] = off
    # the opt-in extensions (no counterpart in the reference): perspective-correct
    # interpolation, bilinear fetch, both; and the transparent pass
    for name, interp, filt in (("ext_perspective", 1, 0), ("ext_bilinear", 0, 1), ("ext_both", 1, 1)):
        d = S.torus_scene(width=160, height=120, nu=24, nv=10, tex=64)
        d.interpolation = interp
        for t in d.textures:
            t.filter = filt
        out[name] = d
    out["transparent"] = cases.transparent_scene()
    return out


def main():
    for name, desc in golden_cases().items():
        bgra, depth, st = oracle_render(desc)
        path = os.path.join(HERE, f"{name}.npz")
        golden_io.save(path, desc, bgra, depth, st)
        print(f"{name}: status {st}, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
