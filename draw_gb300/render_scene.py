"""Renders one of the synthetic workloads a few times on the GPU, for profiling.

    python -m draw_gb300.render_scene headline --frames 3
    python -m draw_gb300.render_scene stress --tris 2000000 --frames 3

headline: the 1920x1080 field of 500 UV spheres (1M triangles, 2048^2 texture,
2 lights); stress: the 3840x2160 micro-sphere field (--tris triangles, default
10M; 4096^2 texture, 4 lights). Each frame is one Scene::render; the last
frame's statistics are printed. --tune sets launch-shape knobs (JSON).
"""
from __future__ import annotations

import argparse
import json
import sys


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m draw_gb300.render_scene")
    ap.add_argument("scene", choices=["headline", "stress"])
    ap.add_argument("--frames", type=int, default=3)
    ap.add_argument("--tris", type=int, default=10_000_000, help="stress: number of triangles")
    ap.add_argument("--tune", default="", help='tuning knobs as JSON, e.g. \'{"small_max_px": 64}\'')
    args = ap.parse_args(argv)

    from . import renderer, scenes

    if args.scene == "headline":
        desc = scenes.sphere_field(width=1920, height=1080, n_spheres=500, slices=50, stacks=21, seed=1234, tex=2048,
                                   n_lights=2)
    else:
        desc = scenes.micro_sphere_field(n_tris=args.tris)
    ctx = renderer.Context(0)
    if args.tune:
        ctx.set_tuning(**json.loads(args.tune))
    b = renderer.build_scene(desc, ctx)
    for _ in range(args.frames):
        b.scene.render(b.canvas)
    ctx.synchronize()
    print(json.dumps({"scene": desc.name, "frames": args.frames, "stats": ctx.last_stats()}))
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
