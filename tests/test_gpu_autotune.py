"""The autotuner: every candidate it times traces the same results, the
plan it returns is usable as trace options, any-hit-only options are not
tried on closest-hit batches, and the N/L search returns a tuned tree."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bvhraytracer_gb300 as pkg  # noqa: E402
from bvhraytracer_gb300 import autotune  # noqa: E402
from bvhraytracer_gb300 import scenes as S  # noqa: E402

from tests import _scenes as TS  # noqa: E402

pytestmark = pytest.mark.gpu

LIGHT = [0.5, 3.0, 0.5]


def _batches(tris, scene, rays):
    d = torch.from_numpy(rays).cuda()
    prims = pkg.hit_prims(scene.trace(d)["hits"].cpu().numpy())
    _, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=4)
    return [(d, "closest"), (torch.from_numpy(ao).cuda(), "any")]


def test_plan_is_valid_and_results_are_unchanged():
    tris, b, _ = TS.bvh("clutter120", 8, 8)
    scene = pkg.Scene(b)
    batches = _batches(tris, scene, TS.clutter_rays(tris))
    plan, scenes = autotune.tune_scene(b, batches, reps=1, scenes={("fp32", 0): scene})
    assert len(plan.choices) == 2
    for (lay, opts, ms), (rays, kind) in zip(plan.choices, batches):
        assert ms > 0 and lay in scenes
        if kind == "closest":
            assert not opts.get("any_order")
        ref = scene.trace(rays, kind=kind)
        got = scenes[lay].trace(rays, kind=kind, **opts)
        key = "hits" if kind == "closest" else "occluded"
        assert torch.equal(got[key].view(torch.uint8), ref[key].view(torch.uint8))
    # every timed candidate is in the table; none for any-hit-only options on closest rays
    assert all(not (k[0] == 0 and dict(k[2]).get("any_order")) for k in plan.table)
    assert len(plan.describe()) == 2


def test_branching_search():
    tris = S.clutter(60, seed=4)
    rays = S.clutter_camera(60, 64, 48, seed=4)

    def batches_fn(scene):
        return _batches(tris, scene, rays)

    best, results = autotune.tune_branching(tris, batches_fn, pairs=((4, 4), (8, 8)), reps=1,
                                            layouts=(("fp32", 0),),
                                            options=({"scheme": "per_ray"},
                                                     {"scheme": "persistent", "policy": 2,
                                                      "refill": 16}))
    total, pair, bvh, plan, scenes = best
    assert pair in ((4, 4), (8, 8)) and set(results) == {(4, 4), (8, 8)}
    assert total == min(results.values())
    assert bvh.info["branching"] == pair[0]


def test_branching_search_keeps_the_preferred_pair_within_the_margin():
    tris = S.clutter(60, seed=4)
    rays = S.clutter_camera(60, 64, 48, seed=4)
    fake = {4: 1.0, 8: 1.04}  # milliseconds by node width: N4 4 % faster

    def batches_fn(scene):
        return _batches(tris, scene, rays)

    def time_fn(scene, batches):
        return fake[scene.bvh_info["branching"]]

    kw = dict(pairs=((4, 4), (8, 8)), layouts=(("fp32", 0),), time_fn=time_fn)
    best, results = autotune.tune_branching(tris, batches_fn, prefer=(8, 8), margin=0.05, **kw)
    assert best[1] == (8, 8) and results == {(4, 4): 1.0, (8, 8): 1.04}
    best, _ = autotune.tune_branching(tris, batches_fn, prefer=(8, 8), margin=0.02, **kw)
    assert best[1] == (4, 4)
    best, _ = autotune.tune_branching(tris, batches_fn, **kw)
    assert best[1] == (4, 4)
