"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py): the
oracle must reproduce them byte for byte on CPU, and the GPU path through the
C ABI must reproduce them on a GB300."""
import glob
import os

import numpy as np
import pytest

import golden_io
from helpers import compare, describe, gpu_render, oracle_render

FIXTURES = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz")))


def _name(p):
    return os.path.splitext(os.path.basename(p))[0]


def test_fixture_set_present():
    names = {_name(p) for p in FIXTURES}
    assert {"tie_rule", "equal_depth", "clip", "degenerate", "offset_collapse", "texture_range"} <= names


@pytest.mark.parametrize("path", FIXTURES, ids=_name)
def test_oracle_reproduces_golden(path, oracle_lib):
    desc, bgra, depth, status = golden_io.load(path)
    b, d, st = oracle_render(desc)
    assert st == status
    if status == 0:
        assert np.array_equal(b, bgra)
        assert np.array_equal(d.view(np.uint32), depth.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=_name)
def test_gpu_reproduces_golden(path, gpu_ctx):
    desc, bgra, depth, status = golden_io.load(path)
    b, d, st = gpu_render(desc, gpu_ctx)
    assert st == status
    if status == 0:
        p = compare((bgra, depth), (b, d), desc.clear_depth)
        assert p.ok, describe(p)
