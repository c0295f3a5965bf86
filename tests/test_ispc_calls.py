"""The reference's ISPC kernels as single calls (aabbIntersect{N},
triIntersect{L}, triAnyHit{L}): the oracle's restatement against known
answers on the CPU, and the batched GPU entry points against the oracle bit
for bit."""
import numpy as np
import pytest

from oracle import oracle as O

FLT_MAX = np.float32(3.4028235e38)


def fastray(o, d, tmax):
    """FastRay::FastRay (src/fastRay.cpp:3-20): invDirection = 1 / direction,
    FLT_MAX where a component is 0."""
    o = np.asarray(o, np.float32)
    d = np.asarray(d, np.float32)
    inv = np.where(d == 0, FLT_MAX, np.float32(1) / np.where(d == 0, np.float32(1), d))
    return np.concatenate([[np.float32(tmax)], o, inv.astype(np.float32), d]).astype(np.float32)


def leaf_block(tris, l):
    """Leaf block rows of width l (x0 y0 z0 x1 ... z2) from [k, 9] triangles."""
    blk = np.zeros(9 * l, np.float32)
    for j, t in enumerate(tris):
        for r in range(9):
            blk[r * l + j] = t[r]
    return blk


TRI = [0, 0, 0, 1, 0, 0, 0, 1, 0]  # z = 0, legs along x and y


def test_tri_intersect_known_answers():
    down = fastray([0.25, 0.25, 2], [0, 0, -1], 10)
    blk = leaf_block([TRI], 4)
    idx, fr = O.tri_intersect_calls(4, 4, blk, np.array([0]), down[None])
    assert idx[0] == 0 and fr[0, 0] == 2.0
    # beyond tMax, outside the triangle, parallel: no hit, tMax kept
    for r in (fastray([0.25, 0.25, 2], [0, 0, -1], 1.5), fastray([0.8, 0.8, 2], [0, 0, -1], 10),
              fastray([0.25, 0.25, 2], [1, 0, 0], 10)):
        idx, fr = O.tri_intersect_calls(4, 4, blk, np.array([0]), r[None])
        assert idx[0] == -1 and fr[0, 0] == r[0]
    assert O.tri_any_hit_calls(4, blk, np.array([0]), down[None])[0] == 1
    assert O.tri_any_hit_calls(4, blk, np.array([0]), fastray([2, 2, 2], [0, 0, -1], 9)[None])[0] == 0


def test_tri_intersect_gang_tie_rule():
    """Equal t in two lanes: the larger in-leaf index wins; twice in one
    lane (index j and j + gang): the lane keeps its first minimum."""
    down = fastray([0.25, 0.25, 2], [0, 0, -1], 10)
    far = [0, 0, -1, 1, 0, -1, 0, 1, -1]
    blk = leaf_block([far, TRI, TRI, far, far, TRI, far, far], 8)
    idx, fr = O.tri_intersect_calls(8, 4, blk, np.array([0]), down[None])
    assert idx[0] == 2 and fr[0, 0] == 2.0  # lanes 1 and 2 tie (5 is lane 1 again)
    blk = leaf_block([far, TRI, far, far, far, TRI, far, far], 8)
    assert O.tri_intersect_calls(8, 4, blk, np.array([0]), down[None])[0][0] == 1
    assert O.tri_intersect_calls(8, 8, blk, np.array([0]), down[None])[0][0] == 5


def test_aabb_intersect_known_answers():
    b = np.zeros(6 * 4, np.float32)
    boxes = [([0, 0, 0], [1, 1, 0.5]), ([2, 2, 2], [3, 3, 3]), ([0, 0, -1], [1, 1, -0.5]),
             ([-1, -1, 5], [1, 1, 6])]
    for j, (lo, hi) in enumerate(boxes):
        for a in range(3):
            b[a * 4 + j] = lo[a]
            b[(3 + a) * 4 + j] = hi[a]
    r = fastray([0.25, 0.25, 1], [0, 0, -1], 10)  # x, y components 0: invDirection FLT_MAX
    res, dist = O.aabb_intersect_calls(4, b, np.array([0]), r[None], np.full((1, 4), -7, np.float32))
    assert res[0] == 1
    assert dist[0].tolist() == [0.5, -7.0, 1.5, -7.0]
    r2 = fastray([0.25, 0.25, 1], [0, 0, -1], 1.0)  # the third box starts beyond tMax
    res, dist = O.aabb_intersect_calls(4, b, np.array([0]), r2[None], np.full((1, 4), -7, np.float32))
    assert dist[0].tolist() == [0.5, -7.0, -7.0, -7.0]


@pytest.mark.gpu
@pytest.mark.parametrize("n,l", [(4, 4), (8, 8), (12, 12), (16, 16)])
def test_gpu_calls_match_oracle(n, l):
    torch = pytest.importorskip("torch")
    import bvhraytracer_gb300 as pkg
    from bvhraytracer_gb300 import scenes as S
    tris = S.clutter(60, seed=5)
    b = pkg.Bvh(tris, n, l)
    fx = b.export_fast()
    nm, lm = fx["node_memory"], fx["leaf_memory"]
    rng = np.random.default_rng(n * 100 + l)
    count = 20000
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    o = rng.uniform(lo, hi, (count, 3)).astype(np.float32)
    d = rng.normal(size=(count, 3)).astype(np.float32)
    d[::7, 0] = 0
    d[::11, 1] = 0
    fr = np.stack([fastray(o[i], d[i], rng.uniform(0.5, 30)) for i in range(count)])
    n_nodes = fx["bounds"].shape[0]
    noff = (rng.integers(0, n_nodes, count) * 6 * nm).astype(np.uint32)
    n_leaves = fx["tri_points"].shape[0] // (9 * lm)
    loff = (rng.integers(0, n_leaves, count) * 9 * lm).astype(np.uint32)
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    bounds = fx["bounds"].reshape(-1)
    dist0 = np.full((count, nm), -7.0, np.float32)
    ref_res, ref_dist = O.aabb_intersect_calls(nm, bounds, noff, fr, dist0)
    d_dist = dev(dist0)
    got = pkg.aabb_intersect(nm, dev(bounds), dev(noff.view(np.int32)), dev(fr), d_dist)
    assert np.array_equal(got.cpu().numpy(), ref_res)
    assert np.array_equal(d_dist.cpu().numpy().view(np.uint32), ref_dist.view(np.uint32))
    assert 0 < ref_res.sum() < count
    tp = fx["tri_points"]
    for gang in (4, 8):
        ref_idx, ref_fr = O.tri_intersect_calls(lm, gang, tp, loff, fr)
        d_fr = dev(fr)
        got = pkg.tri_intersect(lm, gang, dev(tp), dev(loff.view(np.int32)), d_fr)
        assert np.array_equal(got.cpu().numpy(), ref_idx)
        assert np.array_equal(d_fr.cpu().numpy().view(np.uint32), ref_fr.view(np.uint32))
    ref_any = O.tri_any_hit_calls(lm, tp, loff, fr)
    got = pkg.tri_any_hit(lm, dev(tp), dev(loff.view(np.int32)), dev(fr))
    assert np.array_equal(got.cpu().numpy(), ref_any)
    assert ref_any.sum() > 0
    assert pkg.gang_size() == 4
    with pytest.raises(pkg.BvhgpuError):
        pkg.tri_intersect(6, 4, dev(tp), dev(loff.view(np.int32)), dev(fr))


@pytest.mark.gpu
def test_gpu_tie_rule_cases():
    torch = pytest.importorskip("torch")
    import bvhraytracer_gb300 as pkg
    down = fastray([0.25, 0.25, 2], [0, 0, -1], 10)
    far = [0, 0, -1, 1, 0, -1, 0, 1, -1]
    blk = np.concatenate([leaf_block([far, TRI, TRI, far, far, TRI, far, far], 8),
                          leaf_block([far, TRI, far, far, far, TRI, far, far], 8)])
    ids = np.array([0, 72, 72], np.uint32)
    frs = np.stack([down] * 3)
    for gang, expect in ((4, [2, 1, 1]), (8, [5, 5, 5])):
        d_fr = torch.from_numpy(frs.copy()).cuda()
        got = pkg.tri_intersect(8, gang, torch.from_numpy(blk).cuda(),
                                torch.from_numpy(ids.view(np.int32)).cuda(), d_fr)
        ref, _ = O.tri_intersect_calls(8, gang, blk, ids, frs)
        assert got.cpu().numpy().tolist() == ref.tolist() == expect
        assert np.all(d_fr.cpu().numpy()[:, 0] == 2.0)
