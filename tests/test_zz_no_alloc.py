"""The entry point that allocates nothing (bvhgpu_trace_batches_noalloc).

It serves callers that may not allocate GPU memory while they trace — a
plugin inside a host application that owns the GPU memory budget, or a frame
loop that cannot take the synchronisation an allocation may cause. Its
results must equal the regular entry point's, call after call, although all
calls share one fixed scratch array inside the library. This file is named
to run last, and it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bvhraytracer_gb300 as pkg  # noqa: E402
from bvhraytracer_gb300 import _native as N  # noqa: E402
from bvhraytracer_gb300 import scenes as S  # noqa: E402

pytestmark = pytest.mark.gpu


def _frame():
    tris = S.clutter(120, 3)
    rays = S.clutter_camera(120, 96, 64, seed=3)
    bvh = pkg.Bvh(tris, 8, 8)
    scene = pkg.Scene(bvh)
    d = torch.from_numpy(rays).cuda()
    prims = pkg.hit_prims(scene.trace(d)["hits"].cpu().numpy())
    m, p, n = S.surface(tris, rays, prims)
    ao = S.ao_rays(p, n, 4, 0.1 * S.scene_diagonal(tris), seed=5)
    sh = S.shadow_rays(p, n, S.clutter_viewpoints(120, 3)[2])
    return scene, d, torch.from_numpy(sh).cuda(), torch.from_numpy(ao).cuda()


@pytest.mark.parametrize("profile", ["instrumented", "fast"])
def test_noalloc_matches_regular_entry_point_twice(profile):
    scene, prim, shadow, ao = _frame()
    ref_h = scene.trace(prim, scheme="persistent", profile=profile)["hits"]
    ref_s = scene.trace(shadow, kind="any", scheme="persistent", profile=profile)["occluded"]
    ref_a = scene.trace(ao, kind="any", scheme="per_ray", profile=profile)["occluded"]
    for call in range(2):  # the shared scratch keeps the previous call's contents
        out_h = torch.full_like(ref_h, -7.0)
        out_s = torch.full_like(ref_s, 9)
        out_a = torch.full_like(ref_a, 9)
        scene.trace_batches_noalloc([(prim, "closest", out_h), (shadow, "any", out_s),
                                     (ao, "any", out_a)], profile=profile)
        torch.cuda.synchronize()
        assert torch.equal(out_h.view(torch.int32), ref_h.view(torch.int32)), call
        assert torch.equal(out_s, ref_s), call
        assert torch.equal(out_a, ref_a), call
    scene.status()


def test_noalloc_rejects_more_batches_than_the_scratch_holds():
    scene, prim, _, _ = _frame()
    out = torch.empty((prim.shape[0], 4), dtype=torch.float32, device="cuda")
    with pytest.raises(pkg.BvhgpuError) as e:
        scene.trace_batches_noalloc([(prim, "closest", out)] * 65)
    assert e.value.code == N.ERR_BAD_ARG and "64" in str(e.value)
    # 64 batches fit
    outs = [torch.empty_like(out) for _ in range(64)]
    scene.trace_batches_noalloc([(prim, "closest", o) for o in outs])
    ref = scene.trace(prim)["hits"]
    torch.cuda.synchronize()
    assert all(torch.equal(o.view(torch.int32), ref.view(torch.int32)) for o in outs)


@pytest.mark.parametrize("options", [dict(), dict(profile="fast", policy=2, refill=24,
                                                    any_order=True)])
def test_noalloc_makes_no_allocation(options):
    scene, prim, shadow, _ = _frame()
    out_h = torch.empty((prim.shape[0], 4), dtype=torch.float32, device="cuda")
    out_s = torch.empty(shadow.shape[0], dtype=torch.uint8, device="cuda")
    batches = [(prim, "closest", out_h), (shadow, "any", out_s)]
    # Warm-up with the same options: the scratch address look-up and the
    # first load of each kernel variant these options select.
    scene.trace_batches_noalloc(batches, **options)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        scene.trace_batches_noalloc(batches, **options)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    ref_h = scene.trace(prim, profile=options.get("profile", "instrumented"))["hits"]
    assert torch.equal(out_h.view(torch.int32), ref_h.view(torch.int32))


def test_noalloc_rejects_a_short_result_buffer():
    scene, prim, _, _ = _frame()
    short = torch.empty((prim.shape[0] - 1, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError):
        scene.trace_batches_noalloc([(prim, "closest", short)])
