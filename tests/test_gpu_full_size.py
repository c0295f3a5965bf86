"""Full-size parity on the workloads the bench times.

* The 1M-triangle clutter frame (4,000 objects, N8L8, 1920x1080 primary +
  1 shadow + 8 AO rays per hit), traced with the plan the bench's autotuner
  picks (primary: per-ray with local-memory stacks; shadow: persistent,
  speculative any-hit policy 2, refill 16; AO: persistent policy 2, refill
  24, rays grouped into 6 x 10 x 10 direction bins, child-index push order):
  evenly strided samples of each batch equal the oracle's instrumented
  traversal (CompactNodeManager::intersectImmediately) bit for bit, and every
  AO result equals "closest hit within tMax".
* The 8M-triangle clutter scene (32,000 objects, N8L4) at a reduced ray count:
  FP32 and 8-bit quantised nodes give identical hit and occlusion sets.
"""
from types import SimpleNamespace

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bench  # noqa: E402
import bvhraytracer_gb300 as pkg  # noqa: E402
from bvhraytracer_gb300 import scenes as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

BENCH_PLAN = ({"scheme": "per_ray", "stack": "local"},
              {"scheme": "persistent", "policy": 2, "refill": 16},
              {"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 10,
               "any_order": True})


def _strided(n, k):
    return np.unique(np.linspace(0, n - 1, k).astype(np.int64))


def _bits(h):
    return np.ascontiguousarray(h, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def bench_frame():
    a = SimpleNamespace(objects=4000, branching=8, leaf=8, width=1920, height=1080, ao=8)
    tris, bvh, primary = bench.make_frame(a)
    scene = pkg.Scene(bvh)
    d_p = torch.from_numpy(primary).cuda()
    hits = scene.trace(d_p, **BENCH_PLAN[0])["hits"]
    shadow, ao = bench.secondaries(a, tris, primary, pkg.hit_prims(hits.cpu().numpy()))
    return tris, bvh, scene, primary, shadow, ao, hits


def test_bench_frame_with_the_bench_plan_equals_the_oracle(bench_frame):
    tris, bvh, scene, primary, shadow, ao, hits = bench_frame
    assert bvh.info["n_tris"] == 999744 and ao.shape[0] > 16_000_000
    d_s, d_a = torch.from_numpy(shadow).cuda(), torch.from_numpy(ao).cuda()
    occ_s = scene.trace(d_s, kind="any", **BENCH_PLAN[1])["occluded"].cpu().numpy()
    occ_a = scene.trace(d_a, kind="any", **BENCH_PLAN[2])["occluded"].cpu().numpy()
    # two leaves per lane set aside (policy 3), tested per lane or warp-wide
    # (policy 4): the same occlusion
    for policy in (3, 4):
        occ_c = scene.trace(d_a, kind="any", scheme="persistent", policy=policy, refill=24,
                            reorder=10, any_order=True)["occluded"].cpu().numpy()
        assert np.array_equal(occ_c, occ_a), policy
    scene.status()
    cv = O.CompactView(bvh.export_compact())
    for rays, gpu, shadow_kind in ((primary, hits.cpu().numpy(), False), (shadow, occ_s, True),
                                   (ao, occ_a, True)):
        idx = _strided(rays.shape[0], 24_000)
        ref = O.trace_instrumented(cv, rays[idx], shadow=shadow_kind, counters=False)
        if shadow_kind:
            assert np.array_equal(gpu[idx], ref["occluded"])
        else:
            assert np.array_equal(_bits(gpu[idx]), _bits(ref["hits"]))
    # Every AO ray: occluded exactly when its closest hit lies within tMax.
    close = scene.trace(d_a, scheme="persistent", policy=0)["hits"]
    assert np.array_equal(occ_a.astype(bool), close.view(torch.int32)[:, 0].cpu().numpy() >= 0)


def test_scale8m_fp32_and_q8_nodes_give_identical_hit_sets():
    n_obj = 32000
    tris = S.clutter(n_obj, seed=1)
    bvh = pkg.Bvh(tris, 8, 4)
    assert bvh.info["n_tris"] > 7_900_000
    fp32, q8 = pkg.Scene(bvh), pkg.Scene(bvh, node_format="q8")
    assert q8.node_record_bytes == 80 and fp32.node_record_bytes == 240  # 3x fewer node bytes
    primary = S.clutter_camera(n_obj, 640, 360)
    d_p = torch.from_numpy(primary).cuda()
    h32 = fp32.trace(d_p)["hits"]
    prims = pkg.hit_prims(h32.cpu().numpy())
    m, p, n = S.surface(tris, primary, prims)
    ao = torch.from_numpy(S.ao_rays(p, n, 16, 0.1 * S.scene_diagonal(tris), seed=3)).cuda()
    assert ao.shape[0] > 1_000_000
    for o in ({"scheme": "per_ray"},
              {"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 10,
               "any_order": True}):
        hq = q8.trace(d_p, **o)["hits"]
        assert torch.equal(hq.view(torch.int32), fp32.trace(d_p, **o)["hits"].view(torch.int32))
        assert torch.equal(hq.view(torch.int32), h32.view(torch.int32))
        assert torch.equal(q8.trace(ao, kind="any", **o)["occluded"],
                           fp32.trace(ao, kind="any", **o)["occluded"])
    fp32.status()
    q8.status()
    # A strided sample of the primary hits equals the oracle.
    cv = O.CompactView(bvh.export_compact())
    idx = _strided(primary.shape[0], 8_000)
    ref = O.trace_instrumented(cv, primary[idx], shadow=False, counters=False)
    assert np.array_equal(_bits(h32.cpu().numpy()[idx]), _bits(ref["hits"]))
