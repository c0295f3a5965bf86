"""Failure detection without GPU faults: a capped traversal stack reports
BVHGPU_ERR_STACK_OVERFLOW; a staging wait that nothing completes gives up
after its time limit and reports BVHGPU_ERR_TIMEOUT; the context stays
usable. Plus the FP64 error statement of every closest hit."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bvhraytracer_gb300 as pkg  # noqa: E402
from bvhraytracer_gb300 import _native as N  # noqa: E402
from tests import _scenes as TS  # noqa: E402

pytestmark = pytest.mark.gpu


def _scene(**kw):
    tris, b, cv = TS.bvh("clutter120", 8, 4)
    rays = torch.from_numpy(TS.clutter_rays(tris, res=(64, 48))).cuda()
    return b, pkg.Scene(b, **kw), rays


@pytest.mark.parametrize("scheme", ["per_ray", "stream", "persistent"])
def test_stack_limit_reports_overflow(scheme):
    b, scene, rays = _scene()
    full = scene.trace(rays, scheme=scheme)["hits"]
    scene.set_stack_limit(2)
    capped = scene.trace(rays, scheme=scheme)["hits"]
    with pytest.raises(pkg.BvhgpuError) as e:
        scene.status()
    assert e.value.code == N.ERR_STACK_OVERFLOW
    scene.status()  # cleared by the read
    prim_c = capped.view(torch.int32)[:, 0]
    prim_f = full.view(torch.int32)[:, 0]
    # every ray either overflowed (miss) or finished exactly as without the cap
    same = (capped.view(torch.int32) == full.view(torch.int32)).all(1)
    assert bool(((prim_c == -1) | same).all())
    scene.set_stack_limit(0)
    again = scene.trace(rays, scheme=scheme)["hits"]
    assert torch.equal(again.view(torch.int32), full.view(torch.int32))
    scene.status()


def test_staging_wait_times_out_and_context_survives():
    b, scene, rays = _scene(top_levels=2)
    ref = scene.trace(rays, scheme="persistent")["hits"]
    N.check(N.lib().bvhgpu_scene_inject_stall(scene.handle, 1))
    scene.trace(rays, scheme="persistent")
    with pytest.raises(pkg.BvhgpuError) as e:
        scene.status()
    assert e.value.code == N.ERR_TIMEOUT
    N.check(N.lib().bvhgpu_scene_inject_stall(scene.handle, 0))
    again = scene.trace(rays, scheme="persistent")["hits"]
    assert torch.equal(again.view(torch.int32), ref.view(torch.int32))
    scene.status()


@pytest.mark.parametrize("profile", ["instrumented", "fast"])
def test_fp64_error_statement(profile):
    b, scene, rays = _scene()
    hits = scene.trace(rays, profile=profile)["hits"]
    chk = scene.fp64_check(rays, hits, profile=profile).cpu().numpy()
    prim = pkg.hit_prims(hits.cpu().numpy())
    assert np.all(np.isnan(chk[prim < 0]))
    h = chk[prim >= 0]
    assert h.shape[0] > 1000
    assert np.nanmax(h[:, 3]) < 1e-4           # relative t error of FP32
    hv = hits.cpu().numpy()[prim >= 0]
    assert np.max(np.abs(hv[:, 2] - h[:, 1])) < 1e-3  # barycentrics
    assert np.max(np.abs(hv[:, 3] - h[:, 2])) < 1e-3
