"""The DRAW_CHECKED build (draw_gb300/_build.py build(checked=True)): its
kernels test the data-dependent indices of their gathers and scatters against
the buffers' sizes and record DG_E_CUDA, skipping the access, where one is out
of range. It stands in for a memory checker on this GPU: rendering the parity
cases, the torus configuration, the 1080p scene of 1M triangles and the
transparent scene through it must raise no error and still match the oracle
(coverage and depth bit-exact, colour within COLOUR_TOL_LSB).

The checked library is loaded in a child process (DRAW_GB300_LIB), so the
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
import cases
from draw_gb300 import renderer, scenes as S
from helpers import compare, describe, gpu_render, oracle_render
ctx = renderer.Context(0)
descs = {name: fn() for name, fn in sorted(cases.PARITY_CASES.items())}
descs["torus_config"] = S.torus_scene()
descs["sphere_field_full"] = S.sphere_field()
descs["transparent"] = cases.transparent_scene()
out = {}
for name, d in descs.items():
    ref = oracle_render(d)
    got = gpu_render(d, ctx)
    st = got[2]
    p = compare(ref, got, d.clear_depth) if st == 0 else None
    out[name] = dict(status=st, ok=bool(p and p.ok), desc=describe(p) if p else "")
ctx.close()
print(json.dumps(out))
"""


def test_checked_build_renders_parity_cases(oracle_lib):
    from draw_gb300 import _build

    lib = _build.build(checked=True)
    env = dict(os.environ, DRAW_GB300_LIB=lib)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    bad = {k: v for k, v in res.items() if v["status"] != 0 or not v["ok"]}
    assert not bad, bad
    assert len(res) >= 10
