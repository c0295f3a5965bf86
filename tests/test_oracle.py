"""The CPU oracle pinned by known-answer tests: analytic hits, hand-counted
traversals on a hand-built tree, the two tie rules, and stream == per-ray."""
import numpy as np
import pytest

from bvhraytracer_gb300 import scenes as S
from oracle import oracle as O
from tests import _scenes as TS

INF = 222222.0


def ray(o, d, tmax=INF):
    return np.array([[*o, tmax, *d, 0.0]], np.float32)


def tri_at(x, z=5.0):
    return [x, 0, z, x + 1, 0, z, x, 1, z]


def compact_from(nodes, tris):
    """Compact view from a hand-written tree: nodes = list of
    (child_begin, child_count, prim_begin, prim_count, depth)."""
    n = len(nodes)
    t = np.array(tris, np.float32).reshape(-1, 9)
    c = {k: np.zeros(n, np.uint32) for k in ("child_begin", "child_count", "prim_begin", "prim_count")}
    c["depth"] = np.array([x[4] for x in nodes], np.uint8)
    for i, (cb, cc, pb, pc, _) in enumerate(nodes):
        c["child_begin"][i], c["child_count"][i], c["prim_begin"][i], c["prim_count"][i] = cb, cc, pb, pc
    lo = np.zeros((n, 3), np.float32)
    hi = np.zeros((n, 3), np.float32)

    def box(i):
        cb, cc, pb, pc, _ = nodes[i]
        if cc == 0:
            p = t[pb:pb + pc].reshape(-1, 3)
            lo[i], hi[i] = p.min(0), p.max(0)
        else:
            for j in range(cb, cb + cc):
                box(j)
            lo[i] = lo[cb:cb + cc].min(0)
            hi[i] = hi[cb:cb + cc].max(0)

    box(0)
    order = np.zeros((n, 48), np.int8)
    for i, (cb, cc, _, _, _) in enumerate(nodes):
        for a in range(3):
            cen = (hi[cb:cb + cc, a] + lo[cb:cb + cc, a]) + np.float32(0.5)
            order[i, a * 16:a * 16 + cc] = sorted(range(cc), key=lambda j: (cen[j], j))
    c.update(lo3=lo, hi3=hi, order48=order, prim_ids=np.arange(t.shape[0], dtype=np.uint32),
             prim_tri9=t)
    return c


def fast_from(c, gang=4):
    """FastNodeManager arrays for a compact view (fastNodeManager.h:1495-1673)."""
    n = c["child_count"].shape[0]
    nm = max(gang, -(-int(c["child_count"].max()) // gang) * gang)
    lm = max(gang, -(-int(c["prim_count"].max()) // gang) * gang)
    bounds = np.zeros((n, 6 * nm), np.float32)
    begin = np.zeros(n, np.uint32)
    order = np.zeros((n, 3 * nm), np.int8)
    ctype = np.zeros(n, np.uint32)
    tp = []
    for i in range(n):
        cc, pc = int(c["child_count"][i]), int(c["prim_count"][i])
        if cc:
            real = -(-cc // gang) * gang
            ch = np.arange(c["child_begin"][i], c["child_begin"][i] + cc)
            for a in range(3):
                bounds[i, a * real:a * real + cc] = c["lo3"][ch, a]
                bounds[i, 3 * real + a * real:3 * real + a * real + cc] = c["hi3"][ch, a]
            if real != nm:
                bounds[i, -2], bounds[i, -1] = real, np.nan
            begin[i] = c["child_begin"][i]
            ctype[i] = sum(1 << j for j, x in enumerate(ch) if c["child_count"][x] > 0)
            for a in range(3):
                order[i, a * nm:a * nm + cc] = c["order48"][i, a * 16:a * 16 + cc]
        else:
            real = -(-pc // gang) * gang
            blk = np.zeros(lm * 9, np.float32)
            pts = c["prim_tri9"][c["prim_begin"][i]:c["prim_begin"][i] + pc]
            for r in range(9):
                blk[r * real:r * real + pc] = pts[:, r]
            if real != lm:
                blk[-2], blk[-1] = real, np.nan
            begin[i] = len(tp)
            tp.extend(blk.tolist())
            bounds[i, 0] = np.nan
    return {"gang": gang, "node_memory": nm, "leaf_memory": lm, "bounds": bounds, "begin": begin,
            "order": order, "child_type": ctype, "tri_points": np.array(tp, np.float32)}


# Root -> two inner nodes -> two leaves each; one unit triangle per leaf at
# x = 0, 2, 4, 6 in the plane z = 5.
TWO_LEVEL = [(1, 2, 0, 0, 0), (3, 2, 0, 0, 1), (5, 2, 0, 0, 1),
             (0, 0, 0, 1, 2), (0, 0, 1, 1, 2), (0, 0, 2, 1, 2), (0, 0, 3, 1, 2)]
TWO_LEVEL_TRIS = [tri_at(0), tri_at(2), tri_at(4), tri_at(6)]


def views(nodes, tris, gang=4):
    c = compact_from(nodes, tris)
    return O.CompactView(c), O.FastView(fast_from(c, gang))


@pytest.mark.parametrize("packet", [0, 64])
def test_kat_two_level_instrumented(packet):
    cv, _ = views(TWO_LEVEL, TWO_LEVEL_TRIS)
    r = O.trace_instrumented(cv, ray((0.25, 0.25, 0), (0, 0, 1)), shadow=False, packet=packet)
    h = r["hits"][0]
    assert h.view(np.int32)[0] == 0
    assert (h[1], h[2], h[3]) == (5.0, 0.25, 0.25)
    # root + node 1 visited; 4 box tests (2 hit); leaf 3 visited, 1 triangle hit
    assert r["counters"][0].tolist() == [2, 1, 4, 2, 1, 1, 1, 0]
    assert r["depth_hist"][0, :3].tolist() == [1, 1, 0]
    assert r["depth_hist"][1, :3].tolist() == [0, 0, 1]


@pytest.mark.parametrize("packet", [0, 64])
def test_kat_two_level_fast(packet):
    cv, fv = views(TWO_LEVEL, TWO_LEVEL_TRIS)
    r = O.trace_fast(fv, cv, ray((4.25, 0.5, 0), (0, 0, 2)), any_hit=False, packet=packet)
    h = r["hits"][0]
    assert h.view(np.int32)[0] == 2
    # un-normalised direction: t in units of |d| = 2
    assert (h[1], h[2], h[3]) == (2.5, 0.25, 0.5)
    assert r["leaf_index"][0] == 2 * 36 and r["tri_index"][0] == 0
    assert r["counters"][0].tolist() == [2, 1, 4, 2, 1, 1, 1, 0]


def test_kat_miss_and_shadow_limits():
    cv, fv = views(TWO_LEVEL, TWO_LEVEL_TRIS)
    r = O.trace_instrumented(cv, ray((1.5, 0.5, 0), (0, 0, 1)), shadow=False)
    assert r["hits"][0].view(np.int32)[0] == -1 and r["hits"][0][1] == np.float32(INF)
    s = O.trace_instrumented(cv, np.concatenate([ray((0.2, 0.2, 0), (0, 0, 1), 4.9),
                                                 ray((0.2, 0.2, 0), (0, 0, 1), 5.1)]), shadow=True)
    assert s["occluded"].tolist() == [0, 1]
    f = O.trace_fast(fv, cv, np.concatenate([ray((0.2, 0.2, 0), (0, 0, 1), 4.9),
                                            ray((0.2, 0.2, 0), (0, 0, 1), 5.1)]), any_hit=True)
    assert f["occluded"].tolist() == [0, 1]


def test_kat_instrumented_tie_last_visited_wins():
    # One leaf holding the same triangle twice: equal t, the later one wins
    # (each accepted triangle overwrites the hit, triangle.cpp:243).
    cv, _ = views([(0, 0, 0, 2, 0)], [tri_at(0), tri_at(0)])
    r = O.trace_instrumented(cv, ray((0.25, 0.25, 0), (0, 0, 1)), shadow=False)
    assert r["hits"][0].view(np.int32)[0] == 1


def test_kat_shared_edge_uses_double_fallback():
    # Two triangles sharing the edge x + y = 1 (z = 5); a ray through the edge
    # has a zero edge function in both; both are accepted, the later one wins.
    a = [0, 0, 5, 1, 0, 5, 0, 1, 5]
    b = [1, 0, 5, 1, 1, 5, 0, 1, 5]
    cv, _ = views([(0, 0, 0, 2, 0)], [a, b])
    r = O.trace_instrumented(cv, ray((0.5, 0.5, 0), (0, 0, 1)), shadow=False)
    assert r["hits"][0].view(np.int32)[0] == 1
    assert r["counters"][0][5] == 2  # both triangles hit
    cv2, _ = views([(0, 0, 0, 2, 0)], [b, a])
    r2 = O.trace_instrumented(cv2, ray((0.5, 0.5, 0), (0, 0, 1)), shadow=False)
    assert r2["hits"][0].view(np.int32)[0] == 1


@pytest.mark.parametrize("dups,winner", [((1, 5), 1), ((1, 6), 6), ((2, 3), 3), ((0, 4), 0),
                                         ((3, 7), 3), ((0, 1, 4), 1)])
def test_kat_fast_gang_lane_tie_rule(dups, winner):
    # triIntersect{8} with gang 4: lane i % 4 keeps its first minimum; the
    # largest index among lanes at the leaf minimum wins.
    tris = [tri_at(10 + 3 * k) for k in range(8)]
    for d in dups:
        tris[d] = tri_at(0)
    cv, fv = views([(0, 0, 0, 8, 0)], tris)
    r = O.trace_fast(fv, cv, ray((0.25, 0.25, 0), (0, 0, 1)), any_hit=False)
    assert r["tri_index"][0] == winner
    assert r["hits"][0].view(np.int32)[0] == winner


def test_kat_fast_later_leaf_with_equal_t_wins():
    # Across leaves only t > tMax is rejected, so a later leaf with the same t
    # replaces the hit. With equal centres the order is (0, 1); a ray along
    # +z pushes it in reverse, so child 0 is popped first and child 1 last.
    cv, fv = views([(1, 2, 0, 0, 0), (0, 0, 0, 1, 1), (0, 0, 1, 1, 1)], [tri_at(0), tri_at(0)])
    r = O.trace_fast(fv, cv, ray((0.25, 0.25, 0), (0, 0, 1)), any_hit=False)
    assert r["hits"][0].view(np.int32)[0] == 1
    r = O.trace_fast(fv, cv, ray((0.25, 0.25, 9), (0, 0, -1)), any_hit=False)
    assert r["hits"][0].view(np.int32)[0] == 0


@pytest.mark.parametrize("kind", ["terrain", "clutter120"])
@pytest.mark.parametrize("n,l", [(4, 4), (8, 8), (16, 4)])
def test_stream_equals_per_ray(kind, n, l):
    tris, b, cv = TS.bvh(kind, n, l)
    rays = TS.terrain_case()[1][::7] if kind == "terrain" else TS.clutter_rays(tris)
    fv = O.FastView(b.export_fast())
    a = O.trace_instrumented(cv, rays, False)
    s = O.trace_instrumented(cv, rays, False, packet=256)
    for k in ("hits", "counters", "depth_hist"):
        assert np.array_equal(a[k].view(np.uint32), s[k].view(np.uint32)), k
    prims = a["hits"].view(np.int32)[:, 0]
    sh, ao = TS.secondary(tris, rays, prims, [2.0, 3.0, 2.0])
    for sec in (sh, ao):
        a = O.trace_instrumented(cv, sec, True)
        s = O.trace_instrumented(cv, sec, True, packet=64)
        assert np.array_equal(a["occluded"], s["occluded"])
        assert np.array_equal(a["counters"], s["counters"])
        fa = O.trace_fast(fv, cv, sec, True)
        fs = O.trace_fast(fv, cv, sec, True, packet=256)
        assert np.array_equal(fa["occluded"], fs["occluded"])
        assert np.array_equal(fa["counters"], fs["counters"])
        # hit / miss of any-hit rays does not depend on the leaf test
        assert np.mean(fa["occluded"] == a["occluded"]) > 0.999
    fa = O.trace_fast(fv, cv, rays, False)
    fs = O.trace_fast(fv, cv, rays, False, packet=256)
    assert np.array_equal(fa["hits"].view(np.uint32), fs["hits"].view(np.uint32))


def test_any_hit_agrees_with_closest_hit_within_tmax():
    tris, b, cv = TS.bvh("clutter120", 8, 8)
    rays = TS.clutter_rays(tris)
    prims = O.trace_instrumented(cv, rays, False)["hits"].view(np.int32)[:, 0]
    _, ao = TS.secondary(tris, rays, prims, [2, 3, 2])
    occ = O.trace_instrumented(cv, ao, True)["occluded"]
    close = O.trace_instrumented(cv, ao, False)["hits"].view(np.int32)[:, 0]
    assert np.array_equal(occ.astype(bool), close >= 0)


def test_fp64_pairs_error_is_small():
    tris, b, cv = TS.bvh("terrain", 4, 4)
    rays = TS.terrain_case()[1][::5]
    h = O.trace_instrumented(cv, rays, False)["hits"]
    prims = h.view(np.int32)[:, 0]
    m = prims >= 0
    ref = O.fp64_pairs(rays[m], tris[prims[m]], normalise=True)
    rel = np.abs(h[m, 1] - ref[:, 0]) / np.abs(ref[:, 0])
    assert np.nanmax(rel) < 1e-5


def test_scenes_sizes():
    assert S.terrain().shape == (32768, 9)
    assert TS.terrain_case()[1].shape == (512 * 512, 8)
    assert S._uv_sphere(np.zeros(3), 1.0).shape == (256, 9)
    assert S._box(np.zeros(3), np.ones(3)).shape == (192, 9)


# Root with two leaf children on the z axis: a triangle at z = 5 and one at
# z = 8 behind it.
NEAR_FAR = [(1, 2, 0, 0, 0), (0, 0, 0, 1, 1), (0, 0, 1, 1, 1)]
NEAR_FAR_TRIS = [tri_at(0, 5.0), tri_at(0, 8.0)]


@pytest.mark.parametrize("profile", ["instrumented", "fast"])
def test_kat_save_distance_skips_far_leaf(profile):
    # A ray along +z pops the near leaf first (hit at t = 5, tMax = 5); the far
    # leaf was pushed with entry distance 8 > 5, so the save-distance traversal
    # drops it uncounted (intersectSaveDistance, fastNodeManager.h:1256-1259;
    # compactNode.cpp:637-645). The plain traversal visits and tests it.
    cv, fv = views(NEAR_FAR, NEAR_FAR_TRIS)
    r = ray((0.25, 0.25, 0), (0, 0, 1))

    def run(dist):
        if profile == "instrumented":
            return O.trace_instrumented(cv, r, False, use_distance=dist)
        return O.trace_fast(fv, cv, r, False, use_distance=dist)

    plain, dist = run(False), run(True)
    for res in (plain, dist):
        assert res["hits"][0].view(np.int32)[0] == 0 and res["hits"][0][1] == 5.0
    assert plain["counters"][0].tolist() == [1, 2, 2, 2, 2, 1, 2, 0]
    assert dist["counters"][0].tolist() == [1, 1, 2, 2, 1, 1, 2, 0]
    # from the far side the far leaf is near: nothing is skipped
    back = ray((0.25, 0.25, 10), (0, 0, -1))
    b = (O.trace_instrumented(cv, back, False, use_distance=True) if profile == "instrumented"
         else O.trace_fast(fv, cv, back, False, use_distance=True))
    assert b["hits"][0].view(np.int32)[0] == 1 and b["counters"][0][1] == 1


@pytest.mark.parametrize("n,l", [(4, 4), (8, 8)])
def test_save_distance_same_hits_fewer_visits(n, l):
    tris, b, cv = TS.bvh("clutter120", n, l)
    fv = O.FastView(b.export_fast())
    rays = TS.clutter_rays(tris)
    for run in (lambda d: O.trace_instrumented(cv, rays, False, use_distance=d),
                lambda d: O.trace_fast(fv, cv, rays, False, use_distance=d)):
        p, d = run(False), run(True)
        assert np.array_equal(p["hits"].view(np.uint32), d["hits"].view(np.uint32))
        assert np.all(d["counters"][:, 0] <= p["counters"][:, 0])
        assert np.all(d["counters"][:, 1] <= p["counters"][:, 1])
        assert d["counters"][:, 1].sum() < p["counters"][:, 1].sum()
    with pytest.raises(ValueError):
        O.trace_instrumented(cv, rays, False, packet=64, use_distance=True)
