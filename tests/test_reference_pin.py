"""The oracle and the host builder pinned against the reference's own code.

oracle/ref/build_ref.py compiles the reference's SAH builder and instrumented
traversal (src/accelerationStructure/{aabb,node,bvh,compactNode}.cpp,
src/primitives/triangle.cpp, src/ray.cpp) with a GLM stand-in. These tests
need the reference's sources and are skipped where they are absent; the
committed fixtures of tests/golden/ carry the same checks to every machine
(tests/test_golden.py, tests/test_gpu_golden.py).

* The builders (csrc/bvh_builder.cpp, and oracle/sah_builder.c that the CPU
  baseline uses): node for node the reference's tree
  (bounds, children, primitive ranges, per-axis push sequences, depths,
  primitive order) on scenes whose triangle centres are distinct per axis.
  Where centres tie, the reference's unstable std::sort and this builder's
  stable sort may order tied triangles differently.
* The oracle (oracle/bvh_oracle.c), traversing the reference's own tree: hit
  triangle, t, hit point, occlusion, the six per-ray counters, per-depth
  node / leaf visits and the fullness histograms equal the reference's
  CompactNodeManager::intersectImmediately (with and without useDistance) and
  intersectWideAlternative (with its per-step workgroup data), ray for ray.
"""
import numpy as np
import pytest

import bvhraytracer_gb300 as pkg
from bvhraytracer_gb300 import scenes as S
from oracle import oracle as O
from oracle.ref import build_ref
from tests import _scenes as TS

pytestmark = pytest.mark.skipif(not build_ref.available(),
                                reason="the reference's sources are not present")

TREE = ("lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "depth",
        "prim_ids")


@pytest.fixture(scope="module")
def R():
    from oracle.ref import reference
    return reference


def _soup(n=3000, seed=1):
    """Random triangles whose centres are distinct per axis."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0, 10, (n, 1, 3)).astype(np.float32)
    return (c + rng.normal(0, 0.25, (n, 3, 3))).astype(np.float32).reshape(-1, 9)


def _same_tree(ref, ours):
    for k in TREE:
        assert np.array_equal(ref[k], ours[k]), k
    # push sequences: the first child_count entries of each axis
    cc = ref["child_count"]
    o_r = ref["order48"].reshape(-1, 3, 16)
    o_o = ours["order48"].reshape(-1, 3, 16)
    for i in np.nonzero(cc)[0]:
        assert np.array_equal(o_r[i, :, :cc[i]], o_o[i, :, :cc[i]]), i


@pytest.mark.parametrize("n,l", [(2, 1), (4, 4), (8, 8), (16, 16), (3, 5), (12, 2), (5, 13)])
def test_builder_equals_the_reference_builder(R, n, l):
    tris = _soup()
    ref = R.ReferenceBvh(tris, n, l, pkg.sah_factor(n, l))
    ours = pkg.Bvh(tris, n, l)
    assert ours.info["n_nodes"] == ref.n_nodes
    _same_tree(ref.export_compact(), ours.export_compact())
    # the oracle's C builder (the CPU baseline's tree) as well
    _same_tree(ref.export_compact(), O.build_tree(tris, n, l))


@pytest.mark.parametrize("split", [0, 1, 2])
def test_builder_leaf_split_options(R, split):
    tris = _soup(1500, seed=4)
    ref = R.ReferenceBvh(tris, 4, 6, pkg.sah_factor(4, 6), leaf_split_option=split)
    ours = pkg.Bvh(tris, 4, 6, leaf_split_option=split)
    _same_tree(ref.export_compact(), ours.export_compact())


def _check(R, tris, rays, n, l, shadow, *, packet=0, use_distance=False):
    ref = R.ReferenceBvh(tris, n, l, pkg.sah_factor(n, l))
    cv = O.CompactView(ref.export_compact())
    r = ref.trace(rays, shadow, packet=packet, use_distance=use_distance,
                  step_cap=512 if packet else 0)
    if packet:
        o = O.trace_instrumented_steps(cv, rays, shadow, packet, 512)
        assert np.array_equal(o["step_count"], r["step_count"])
        assert np.array_equal(o["steps"], r["steps"])
    else:
        o = O.trace_instrumented(cv, rays, shadow=shadow, use_distance=use_distance)
    if shadow:
        assert np.array_equal(o["occluded"], r["occluded"])
    else:
        prim = o["hits"].view(np.int32)[:, 0]
        hit = prim >= 0
        if not packet:
            assert np.array_equal(prim, r["prim"])
        assert np.array_equal(hit, ~np.isnan(r["pos"][:, 0]))
        assert np.array_equal(o["hits"][hit, 1].view(np.uint32), r["t"][hit].view(np.uint32))
        pos = O.hit_points(rays[hit], tris[prim[hit]])
        assert np.array_equal(pos.view(np.uint32), r["pos"][hit].view(np.uint32))
    assert np.array_equal(o["counters"][:, :6], r["counters"])
    assert np.array_equal(o["depth_hist"], r["depth_hist"])
    assert np.array_equal(o["fullness"][0, :n + 1], r["child_fullness"])
    assert np.array_equal(o["fullness"][1, :l + 1], r["prim_fullness"])
    return o


def test_terrain_primary_rays(R):
    tris, rays, light = TS.terrain_case()
    _check(R, tris, rays[::4], 4, 4, False)
    _check(R, tris, rays[::16], 4, 4, False, use_distance=True)
    _check(R, tris, rays[:8192], 4, 4, False, packet=256)


@pytest.mark.parametrize("n,l", [(8, 8), (4, 16), (16, 4), (3, 5), (2, 1)])
def test_clutter_primary_shadow_and_ao_rays(R, n, l):
    tris = TS.clutter_tris(120)
    rays = TS.clutter_rays(tris)
    o = _check(R, tris, rays, n, l, False)
    prim = o["hits"].view(np.int32)[:, 0]
    sh, ao = TS.secondary(tris, rays, prim, [2.0, 3.0, 2.0], ao_samples=2)
    _check(R, tris, sh, n, l, True)
    _check(R, tris, ao, n, l, True)
    _check(R, tris, ao[:4096], n, l, True, packet=256)


def test_edge_case_rays(R):
    """Zero direction components, rays along the axes, NaN, infinite, zero
    and negative tMax, rays starting inside objects."""
    tris = TS.clutter_tris(120)
    rng = np.random.default_rng(9)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    n = 4096
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(lo, hi, (n, 3))
    rays[:, 4:7] = rng.normal(0, 1, (n, 3))
    rays[:, 3] = 1e3
    rays[0::7, 4] = 0
    rays[1::7, 4:6] = 0
    rays[2::11, 3] = np.inf
    rays[3::13, 3] = 0
    rays[4::17, 3] = -1
    rays[5::19, 3] = np.nan
    rays[6::23, 4:7] = [0, 0, -1]
    for n_, l_ in ((8, 8), (4, 4)):
        _check(R, tris, rays, n_, l_, False)
        _check(R, tris, rays, n_, l_, True)


def test_terrain_workload_tree_matches_when_centres_do_not_tie(R):
    """The small configuration's terrain (48 x 48 quads here) with each
    triangle moved by its own small offset, so that no two triangle centres
    tie on an axis (checked)."""
    tris = S.terrain(48, seed=0).reshape(-1, 3, 3)
    i = np.arange(tris.shape[0], dtype=np.float32)[:, None, None]
    tris = (tris + i * np.float32(5e-7) * np.array([1.0, 1.3, 0.7], np.float32)).astype(np.float32)
    c = tris.max(1) * np.float32(0.5) + tris.min(1) * np.float32(0.5)
    assert all(np.unique(c[:, a]).size == c.shape[0] for a in range(3))
    tris = tris.reshape(-1, 9)
    for n, l in ((4, 4), (8, 8)):
        ref = R.ReferenceBvh(tris, n, l, pkg.sah_factor(n, l))
        _same_tree(ref.export_compact(), pkg.Bvh(tris, n, l).export_compact())
