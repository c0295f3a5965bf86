"""The ray-generation restatement (oracle/raygen_ref.py) pinned on the CPU:
FNV-1a test vectors, exact float32 rounding of 64-bit hashes, the camera
against the float64 host generator, and the geometry of secondary rays."""
import numpy as np

import bvhraytracer_gb300 as pkg
from bvhraytracer_gb300 import scenes as S
from oracle import raygen_ref as R


def test_fnv1a64_published_vectors():
    # FNV-1a 64-bit test vectors of the algorithm's authors.
    assert R.fnv1a64_bytes(b"") == 0xCBF29CE484222325
    assert R.fnv1a64_bytes(b"a") == 0xAF63DC4C8601EC8C
    assert R.fnv1a64_bytes(b"foobar") == 0x85944171F73967E8
    assert R.fnv1a64_u64(0x61) == R.fnv1a64_bytes(b"a" + bytes(7))


def test_u64_to_float_rounds_to_nearest_even():
    assert R.u64_to_f32(2 ** 24 + 1) == np.float32(2 ** 24)
    assert R.u64_to_f32(2 ** 24 + 3) == np.float32(2 ** 24 + 4)
    assert R.u64_to_f32(2 ** 64 - 1) == np.float32(2.0 ** 64)
    for x in (12345, 2 ** 40 + 7, 2 ** 63 + 2 ** 38 + 1):
        assert abs(float(R.u64_to_f32(x)) - x) <= 2.0 ** (x.bit_length() - 25)


def test_camera_matches_host_generator():
    pos, target = [0.3, 1.2, 2.0], [0.5, 0.0, 0.5]
    m = pkg.camera_transform(pos, target)
    a = R.camera_rays(pos, m, 64, 40, tile=16)
    b = S.camera_rays(pos, target, 64, 40, tile=16)
    assert a.shape == b.shape
    np.testing.assert_allclose(a[:, 4:7], b[:, 4:7], rtol=0, atol=2e-6)
    assert np.array_equal(a[:, 0:4], b[:, 0:4].astype(np.float32))


def test_secondary_geometry():
    tris = np.array([[0, 0, 5, 1, 0, 5, 0, 1, 5]], np.float32)
    prim = np.array([0, -1], np.int32)
    hits = np.zeros((2, 4), np.float32)
    hits.view(np.int32)[:, 0] = prim
    rays = np.array([[0.25, 0.25, 0, 100, 0, 0, 2, 0]] * 2, np.float32)
    sh, ao, n = R.secondary_rays(tris, rays, hits, light=[0.25, 0.25, 10.0], ao_samples=16,
                                 ao_length=0.5, sampling="cosine", seed=3)
    assert np.allclose(n[0], [0, 0, 1]) and np.isnan(n[1]).all()
    assert np.allclose(sh[0, 0:3], [0.25, 0.25, 5.001]) and np.isclose(sh[0, 3], 4.999)
    assert np.allclose(sh[0, 4:7], [0, 0, 1]) and np.isnan(sh[1, 0])
    d = ao[:16, 4:7]
    assert np.allclose(np.linalg.norm(d, axis=1), 1, atol=1e-6) and (d[:, 2] >= 0).all()
    assert np.isnan(ao[16:, 0]).all()
    _, ao_r, _ = R.secondary_rays(tris, rays, hits, ao_samples=8, sampling="reference", seed=7)
    dr = ao_r[:8, 4:7]
    assert np.allclose(np.linalg.norm(dr, axis=1), 1, atol=1e-6) and (dr[:, 2] > 0).all()
    assert np.allclose(R.ao_factor(np.array([1, 0, 0, 1, 1, 1, 1, 1], np.uint8), 4), [0.5, 0.0])
