"""The DRAW_TIMELINE build (draw_gb300/_build.py build(timeline=True),
dg_timeline_read, python -m draw_gb300.timeline): its kernels record block
start, wait and end times in the global timer. Rendering the torus and the
1080p field of 1M triangles through it must give the oracle's frame, and the
records must describe the programmatic dependent launch chain: every kernel
starts before it ends, its waits lie between, and no kernel passes its wait
before the previous kernel's last block has finished.

The timeline library is loaded in a child process (DRAW_GB300_LIB), so the
process running the other tests keeps the normal build."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
from draw_gb300 import renderer, scenes as S
from helpers import compare, describe, oracle_render
ctx = renderer.Context(0)
out = {}
for name, d in [("torus", S.torus_scene()), ("sphere_field", S.sphere_field())]:
    b = renderer.build_scene(d, ctx)
    ctx.timeline()
    b.scene.render(b.canvas)
    tl = ctx.timeline()
    ref = oracle_render(d)
    p = compare(ref, (*b.canvas.read(), 0), d.clear_depth)
    out[name] = dict(ok=bool(p.ok), desc=describe(p), timeline=tl)
ctx.close()
print(json.dumps(out))
"""


def test_timeline_build_renders_and_orders_the_chain(oracle_lib):
    from draw_gb300 import _build, renderer

    lib = _build.build(timeline=True)
    env = dict(os.environ, DRAW_GB300_LIB=lib)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for name, v in res.items():
        assert v["ok"], f"{name}: {v['desc']}"
        tl = v["timeline"]
        prev_end = None
        for k in renderer.KERNELS:
            start, first_wait, last_wait, end = tl[k]
            assert start is not None and end is not None and start <= end, (name, k, tl[k])
            if first_wait is not None:
                assert start <= first_wait <= last_wait <= end, (name, k, tl[k])
                if prev_end is not None:
                    assert first_wait >= prev_end, (name, k, tl)
            prev_end = end
