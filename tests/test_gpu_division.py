"""The raster pass divides a covered pixel's edge values by the triangle's dens
with Markstein's method from per-triangle reciprocals (div_rcp); coverage and
depth stay bit-exact only if that equals IEEE division on every operand pair the
pass admits. dg_check_division runs the comparison on the device."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode,samples", [(0, 4097 * 4097), (1, 1 << 30), (2, 1 << 30), (3, 1 << 30)])
def test_markstein_division_matches_ieee(gpu_ctx, mode, samples):
    n, a, b = gpu_ctx.check_division(mode, samples, seed=12345)
    assert n == 0, f"{n} mismatches; first a={a!r} b={b!r}"


def test_other_seeds(gpu_ctx):
    for seed in (1, 2, 3):
        for mode in (1, 2, 3):
            n, a, b = gpu_ctx.check_division(mode, 1 << 27, seed=seed)
            assert n == 0, f"mode {mode} seed {seed}: {n} mismatches; first a={a!r} b={b!r}"
