"""Kernel timeline of one render job on the GPU, from the DRAW_TIMELINE build
(draw_gb300/_build.py build(timeline=True), dg_timeline_read):

    python -m draw_gb300.timeline headline --frames 20
    python -m draw_gb300.timeline torus
    python -m draw_gb300.timeline stress --tris 2000000

For each kernel of the job, in microseconds after the first k_vertex block
started: when its first block started, when its first and its last block
passed the wait for the previous kernel (programmatic dependent launch), and
when its last block finished. Each frame follows a write of 256 MiB (the L2
flushed, as bench.py times frames); the medians over the frames are printed as
one JSON line. The marks are atomics of thread 0 of every block, so the frame
takes a few microseconds longer than in the normal build.

The process builds the timeline library if needed and runs the measurement in
a child process that loads it (DRAW_GB300_LIB), so the caller's own process
keeps the normal build.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys

SCENES = ["headline", "torus", "stress"]


def _scene(name: str, tris: int):
    from . import scenes

    if name == "headline":
        return scenes.sphere_field()
    if name == "torus":
        return scenes.torus_scene()
    return scenes.micro_sphere_field(n_tris=tris)


def measure(name: str, frames: int = 20, tris: int = 10_000_000) -> dict:
    """The median timeline of `frames` renders of scene `name` (run in a process
    that loaded the DRAW_TIMELINE build)."""
    import torch

    from . import renderer

    ctx = renderer.Context(0)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    b = renderer.build_scene(_scene(name, tris), ctx)
    rows = []
    with torch.cuda.stream(stream):
        for i in range(frames + 3):
            flush.zero_()
            torch.cuda.synchronize()
            ctx.timeline()  # clears the record
            b.scene.render(b.canvas)
            t = ctx.timeline()
            if i >= 3:
                rows.append(t)
    stats = ctx.last_stats()
    ctx.close()
    out = {}
    for k in renderer.KERNELS:
        cols = []
        for j in range(4):
            vals = [r[k][j] for r in rows if r[k][j] is not None]
            cols.append(round(statistics.median(vals), 2) if vals else None)
        out[k] = dict(zip(["start", "first_wait", "last_wait", "end"], cols))
    return {"scene": name, "frames": frames, "timeline_us": out,
            "stats": {k: int(v) for k, v in stats.items()}}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m draw_gb300.timeline")
    ap.add_argument("scene", choices=SCENES)
    ap.add_argument("--frames", type=int, default=20)
    ap.add_argument("--tris", type=int, default=10_000_000, help="stress: number of triangles")
    args = ap.parse_args(argv)
    from . import _build

    lib = _build.TIMELINE_LIB
    if os.environ.get("DRAW_GB300_LIB") != lib:
        _build.build(timeline=True)
        env = dict(os.environ, DRAW_GB300_LIB=lib)
        rest = sys.argv[1:] if argv is None else list(argv)
        root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        return subprocess.run([sys.executable, "-m", "draw_gb300.timeline", *rest], env=env, cwd=root).returncode
    print(json.dumps(measure(args.scene, args.frames, args.tris)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
