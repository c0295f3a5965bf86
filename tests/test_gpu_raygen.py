"""Ray generation on the GPU (bvhgpu_camera_rays, bvhgpu_secondary_rays,
bvhgpu_ao_factor) against the float32 restatement in oracle/raygen_ref.py:
camera rays, ray origins and shadow rays bit for bit; AO directions (built
with sin / cos / acos) to a few ulps."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bvhraytracer_gb300 as pkg  # noqa: E402
from bvhraytracer_gb300 import scenes as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import raygen_ref as R  # noqa: E402
from tests import _scenes as TS  # noqa: E402

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("w,h,tile", [(1920, 1080, 16), (37, 23, 8), (64, 64, 16), (5, 3, 4)])
def test_camera_rays_bit_exact(w, h, tile):
    pos, target = [1.0, 2.0, 3.5], [0.2, 0.1, -0.3]
    got = pkg.camera_rays(pos, target, w, h, workgroup=tile).cpu().numpy()
    ref = R.camera_rays(pos, pkg.camera_transform(pos, target), w, h, tile=tile)
    assert np.array_equal(bits(got), bits(ref))


@pytest.fixture(scope="module")
def frame():
    tris, b, cv = TS.bvh("clutter120", 8, 8)
    cam, target, light = S.clutter_viewpoints(120, seed=3)
    rays = pkg.camera_rays(cam, target, 96, 64)
    scene = pkg.Scene(b)
    hits = scene.trace(rays)["hits"]
    return tris, cv, scene, rays, hits, light


def _close_dirs(got, ref, normals, S):
    g, r = got[:, 4:7], ref[:, 4:7]
    ok = np.all(np.abs(g - r) <= 2e-6, axis=1)
    # a direction within rounding of the tangent plane may be flipped
    n = np.repeat(normals, S, axis=0)
    grazing = np.abs(np.sum(r * n, axis=1)) < 1e-5
    flipped = np.all(np.abs(g + r) <= 2e-6, axis=1) & grazing
    live = ~np.isnan(r[:, 0])
    assert np.all((ok | flipped)[live])


@pytest.mark.parametrize("sampling", ["cosine", "reference"])
def test_secondary_rays_match_restatement(frame, sampling):
    tris, cv, scene, rays, hits, light = frame
    ns = 4
    sh, ao = scene.secondary_rays(rays, hits, light=light, ao_samples=ns, ao_length=0.7,
                                  sampling=sampling, seed=11)
    h = hits.cpu().numpy()
    rs, ra, nrm = R.secondary_rays(tris, rays.cpu().numpy(), h, light=light, ao_samples=ns,
                                   ao_length=0.7, sampling=sampling, seed=11)
    assert np.array_equal(bits(sh.cpu().numpy()), bits(rs))
    a = ao.cpu().numpy()
    assert np.array_equal(bits(a[:, 0:4]), bits(ra[:, 0:4]))
    _close_dirs(a, ra, nrm, ns)
    miss = h.view(np.int32)[:, 0] < 0
    assert np.isnan(a.reshape(-1, ns, 8)[miss, :, 0]).all()


def test_device_frame_pipeline_parity(frame):
    """Camera -> primary -> secondary -> AO, all on the device; the AO
    occlusion equals the oracle's on the same rays, and the AO factor is the
    per-pixel fraction."""
    tris, cv, scene, rays, hits, light = frame
    ns = 8
    _, ao = scene.secondary_rays(rays, hits, ao_samples=ns, ao_length=0.5)
    occ = scene.trace(ao, kind="any", scheme="persistent", policy=2, refill=16, reorder=8)
    occ = occ["occluded"]
    ref = O.trace_instrumented(cv, ao.cpu().numpy(), shadow=True, counters=False)["occluded"]
    assert np.array_equal(occ.cpu().numpy(), ref)
    f = pkg.ao_factor(occ, ns).cpu().numpy()
    assert np.array_equal(f, R.ao_factor(ref, ns))
