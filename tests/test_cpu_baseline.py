"""The timed CPU baseline (oracle/_build/libcpubaseline.so: the fast-profile
restatement with the ISPC gang lanes as 4-wide vectors) returns exactly what
the scalar oracle returns: hits (prim, t, barycentrics), the reference's
(leafIndex, triIndex) encoding, occlusion and counters, for both schemes,
gang 4 and 8, closest and any-hit rays, odd widths and ragged packets."""
import numpy as np
import pytest

import bvhraytracer_gb300 as pkg
from oracle import oracle as O
from tests import _scenes as TS


def _same(a, b):
    for k in ("hits", "occluded", "leaf_index", "tri_index", "counters", "depth_hist"):
        if a[k] is None:
            assert b[k] is None
            continue
        assert np.array_equal(np.ascontiguousarray(a[k]).view(np.uint8),
                              np.ascontiguousarray(b[k]).view(np.uint8)), k


@pytest.mark.parametrize("n,l,gang", [(8, 8, 4), (4, 4, 4), (16, 16, 4), (3, 5, 4), (8, 8, 8),
                                      (12, 7, 8)])
def test_vectorised_baseline_equals_scalar_oracle(n, l, gang):
    tris = TS.clutter_tris(120)
    b = pkg.Bvh(tris, n, l, gang=gang)
    cv = O.CompactView(b.export_compact())
    fv = O.FastView(b.export_fast(gang=gang))
    rays = TS.clutter_rays(tris)[:4000 - 3].copy()
    rays[::97, 4] = 0.0  # zero direction components
    ref = O.trace_fast(fv, cv, rays, any_hit=False)
    prims = ref["hits"].view(np.int32)[:, 0]
    sh, ao = TS.secondary(tris, rays, prims, [2.0, 3.0, 2.0], ao_samples=2)
    for r, any_hit in ((rays, False), (sh, True), (ao, True)):
        for packet in (0, 256):
            a = O.trace_fast(fv, cv, r, any_hit, packet=packet)
            v = O.trace_fast(fv, cv, r, any_hit, packet=packet, baseline=True)
            _same(a, v)
            v2 = O.trace_fast(fv, cv, r, any_hit, packet=packet, baseline=True, counters=False,
                              threads=4)
            assert np.array_equal((v2["occluded"] if any_hit else v2["hits"]).view(np.uint8),
                                  (a["occluded"] if any_hit else a["hits"]).view(np.uint8))


@pytest.mark.parametrize("n,l,gang,split", [(8, 8, 4, 1), (4, 4, 4, 1), (3, 5, 4, 1),
                                            (16, 16, 8, 1), (12, 7, 8, 1), (2, 1, 4, 1),
                                            (4, 6, 4, 0), (4, 6, 4, 2)])
def test_oracle_builder_and_fast_arrays_equal_the_product_ones(n, l, gang, split):
    """oracle/sah_builder.c and oracle.fast_arrays (the reference arm's tree,
    no product code) give the product builder's tree node for node and its
    FastNodeManager export byte for byte, ties in the centre sort included."""
    for tris in (TS.clutter_tris(120), TS.terrain_case()[0]):
        o = O.build_tree(tris, n, l, gang=gang, leaf_split_option=split)
        b = pkg.Bvh(tris, n, l, gang=gang, leaf_split_option=split)
        p = b.export_compact()
        for k in ("lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count",
                  "order48", "depth", "prim_ids", "prim_tri9"):
            assert np.array_equal(o[k], p[k]), k
        assert o["max_stack"] == b.info["max_stack"]
        f, pf = O.fast_arrays(o, gang=gang), b.export_fast(gang=gang)
        for k in ("bounds", "begin", "order", "child_type", "tri_points"):
            assert np.array_equal(np.asarray(f[k]).view(np.uint8), np.asarray(pf[k]).view(np.uint8)), k
