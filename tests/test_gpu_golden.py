"""The CUDA kernels against the golden fixtures of tests/golden/, which the
reference's own code produced (CompactNodeManager<CompactNodeV3> over the
reference's SAH tree; tests/golden/make_golden.py).

Every scheme traverses the reference's tree from the fixture (imported with
bvhgpu_bvh_import_compact) in the instrumented profile, and must return the
reference's hit triangle and t bit for bit, its occlusion results, and, with
counters, its per-ray node / leaf / box / triangle counts, per-depth visits
and fullness histograms. 8-bit quantised nodes keep the same hits.
"""
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bvhraytracer_gb300 as pkg  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = sorted((Path(__file__).resolve().parent / "golden").glob("reference_*.npz"))
TREE = ("lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "order48",
        "prim_ids")
SCHEMES = [("per_ray", {}), ("per_ray", {"stack": "local"}), ("per_ray", {"save_distance": True}),
           ("stream", {}), ("persistent", {"policy": 0}), ("persistent", {"policy": 1, "refill": 1}),
           ("persistent", {"policy": 2, "refill": 24}),
           ("persistent", {"policy": 2, "refill": 24, "reorder": 10}),
           ("persistent", {"policy": 3, "refill": 24, "reorder": 10, "any_order": True}),
           ("persistent", {"policy": 4, "refill": 24}),
           ("persistent", {"policy": 4, "refill": 24, "reorder": 10, "any_order": True})]
IDS = ["per_ray", "per_ray_local", "per_ray_dist", "stream", "ww", "ifif", "spec", "spec_reorder",
       "spec2_reorder_anyorder", "coop", "coop_reorder_anyorder"]


@pytest.fixture(scope="module", params=GOLDEN, ids=[p.stem for p in GOLDEN])
def case(request):
    z = dict(np.load(request.param))
    tree = {k: z[k] for k in TREE}
    tree["prim_tri9"] = z["tris"][z["prim_ids"]]
    bvh = pkg.Bvh.from_compact(tree, int(z["N"]), int(z["L"]))
    return z, bvh, pkg.Scene(bvh)


def _check_results(z, batch, kind, r):
    if kind == "any":
        assert np.array_equal(r["occluded"].cpu().numpy(), z[batch + "_occluded"]), batch
    else:
        h = r["hits"].cpu().numpy()
        prim = h.view(np.int32)[:, 0]
        assert np.array_equal(prim, z[batch + "_prim"]), batch
        hit = prim >= 0
        assert np.array_equal(h[hit, 1].view(np.uint32), z[batch + "_t"][hit].view(np.uint32))


@pytest.mark.parametrize("scheme,kw", SCHEMES, ids=IDS)
def test_kernels_equal_reference_fixture(case, scheme, kw):
    z, bvh, scene = case
    for batch, kind in (("primary", "closest"), ("shadow", "any"), ("ao", "any")):
        if kw.get("save_distance") and kind == "any":
            continue
        rays = torch.from_numpy(z[batch + "_rays"]).cuda()
        # Without counters every option runs its own kernel (with counters the
        # speculative any-hit policies run the counting one). Save-distance
        # skips pops, so its counters are its own (its hits are the
        # reference's); reordered and any_order launches are compared on
        # results.
        r = scene.trace(rays, kind=kind, scheme=scheme, **kw)
        _check_results(z, batch, kind, r)
        counting = not (kw.get("reorder") or kw.get("save_distance") or kw.get("any_order"))
        if not counting:
            continue
        r = scene.trace(rays, kind=kind, scheme=scheme, counters=True, depth_hist=True, **kw)
        _check_results(z, batch, kind, r)
        if counting:
            c = r["counters"].cpu().numpy().astype(np.uint32)[:, :6]
            assert np.array_equal(c, z[batch + "_counters"]), batch
            assert np.array_equal(r["depth_hist"].cpu().numpy().astype(np.uint64),
                                  z[batch + "_depth_hist"]), batch
            assert np.array_equal(r["fullness"].cpu().numpy().astype(np.uint64),
                                  z[batch + "_fullness"]), batch
    scene.status()


def test_q8_nodes_keep_reference_hits(case):
    z, bvh, _ = case
    q8 = pkg.Scene(bvh, node_format="q8", top_levels=2)
    rays = torch.from_numpy(z["primary_rays"]).cuda()
    h = q8.trace(rays, scheme="persistent", policy=2, refill=16)["hits"].cpu().numpy()
    prim = h.view(np.int32)[:, 0]
    assert np.array_equal(prim, z["primary_prim"])
    assert np.array_equal(h[prim >= 0, 1].view(np.uint32),
                          z["primary_t"][prim >= 0].view(np.uint32))
    for batch in ("shadow", "ao"):
        occ = q8.trace(torch.from_numpy(z[batch + "_rays"]).cuda(), kind="any",
                       scheme="persistent", policy=2, refill=24)["occluded"]
        assert np.array_equal(occ.cpu().numpy(), z[batch + "_occluded"]), batch
    q8.status()


def test_stream_step_log_equals_reference(case):
    """The ray-stream kernel's per-step workgroup data of 256-ray packets
    equals intersectWideAlternative's (CameraData's workgroup analysis)."""
    z, bvh, scene = case
    rays = torch.from_numpy(z["wide_rays"]).cuda()
    r = scene.trace(rays, scheme="stream", counters=True, steps=512)
    cnt = r["step_count"].cpu().numpy()
    assert np.array_equal(cnt, z["wide_step_count"])
    st = r["step_stats"].cpu().numpy()
    for p in range(cnt.shape[0]):
        assert np.array_equal(st[p, :cnt[p]], z["wide_steps"][p, :cnt[p]]), p
    assert np.array_equal(r["counters"].cpu().numpy().astype(np.uint32)[:, :6], z["wide_counters"])
