"""CPU tests of the synthetic scene generators used by the parity tests and the bench."""
import hashlib

import numpy as np

from draw_gb300 import scenes as S


def test_texture_is_integer_only_and_stable():
    t = S.value_noise_checker(64, 32, 1234, comps=4)
    assert t.img.dtype == np.uint8 and t.img.size == 64 * 32 * 4
    again = S.value_noise_checker(64, 32, 1234, comps=4)
    assert np.array_equal(t.img, again.img)
    # integer hashing only: the digest is the same on every platform
    assert hashlib.sha256(t.img.tobytes()).hexdigest()[:16] == hashlib.sha256(again.img.tobytes()).hexdigest()[:16]
    assert (t.img.reshape(-1, 4)[:, 3] == 255).all()
    assert S.value_noise_checker(64, 32, 1235).img.tobytes() != t.img.tobytes()


def _front_fraction(pos, tri, cam):
    a, b, c = pos[tri[:, 0]], pos[tri[:, 1]], pos[tri[:, 2]]
    n = np.cross(b - a, c - b)
    ctr = (a + b + c) / 3
    return float(((np.asarray(cam) - ctr) * n).sum(1).__gt__(0).mean())


def test_torus_counts_and_winding():
    pos, nrm, uv, tri = S.torus(1.0, 0.4, 80, 30)
    assert tri.shape == (4800, 3) and pos.shape == (81 * 31, 3)
    # normals point outward along (b-a)x(c-b)
    a, b, c = pos[tri[:, 0]], pos[tri[:, 1]], pos[tri[:, 2]]
    n = np.cross(b - a, c - b)
    assert ((n * nrm[tri[:, 0]]).sum(1) > 0).mean() > 0.99
    assert 0.3 < _front_fraction(pos, tri, (0, 1.5, 2.6)) < 0.7
    assert uv.min() >= 0 and uv.max() <= 1


def test_sphere_counts():
    pos, nrm, uv, tri = S.uv_sphere(1.0, 50, 21)
    assert tri.shape[0] == 2000
    assert np.allclose(np.linalg.norm(pos, axis=1), 1.0, atol=1e-6)


def test_sphere_field_config():
    d = S.sphere_field(width=1920, height=1080)
    assert d.n_tris == 1_000_000
    assert d.objects[0].vertices.shape[0] == 500 * 51 * 22
    assert 0.02 < d.near_crossing < 0.10  # about 5% of the instances cross the near plane
    assert d.textures[0].width == 2048 and len(d.lights) == 2


def test_batch_frames_ranges():
    fr = S.batch_frames(n_frames=12, seed=3, tri_range=(1000, 5000), tex_range=(64, 128))
    assert len(fr) == 12
    for d in fr:
        assert 128 <= d.width <= 512 and d.width == d.height
        assert 500 <= d.n_tris <= 6000
        assert d.textures[0].width in (64, 128)


def test_micro_sphere_field_statistics():
    """Stress config shape on a reduced triangle count: the same sphere size,
    slab and window, so the per-sphere statistics match the full 10M case."""
    d = S.micro_sphere_field(n_tris=400_000, tex=64)
    assert d.n_tris == 400_000 and d.objects[0].vertices.shape[0] == 10_000 * 36
    assert 0.07 < d.near_crossing < 0.13  # about 10% of the spheres cross the near plane
    assert 1.5 < d.mean_tri_px_est < 2.5  # about 2 px per front-facing triangle
    assert len(d.lights) == 4
    full = S.micro_sphere_field.__defaults__
    assert full[0] == 3840 and full[1] == 2160 and full[2] == 10_000_000 and full[6] == 4096
