"""Host SAH builder: node-for-node equality with the independent Python
restatement, structural invariants, and the FastNodeManager export layout."""
import numpy as np
import pytest

import bvhraytracer_gb300 as pkg
from bvhraytracer_gb300 import scenes as S
from oracle import builder_ref as BR


def _small(kind):
    return S.terrain(10, 4) if kind == "terrain" else S.clutter(4, 6)


@pytest.mark.parametrize("kind", ["terrain", "clutter"])
@pytest.mark.parametrize("n,l,opt", [(4, 4, 1), (8, 8, 1), (16, 4, 1), (12, 16, 1), (2, 1, 1),
                                     (5, 3, 1), (4, 4, 0), (8, 4, 2), (16, 16, 0)])
def test_matches_python_restatement(kind, n, l, opt):
    tris = _small(kind)
    b = pkg.Bvh(tris, n, l, leaf_split_option=opt)
    got = b.export_compact()
    ref = BR.build(tris, n, l, b.params.sah_factor, leaf_split_option=opt)
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k


def _invariants(b: pkg.Bvh, tris):
    c = b.export_compact()
    n, l = b.info["branching"], b.info["leaf_size"]
    cc, pc = c["child_count"], c["prim_count"]
    assert np.all((cc == 0) != (pc == 0)), "a node is exactly one of inner / leaf"
    inner = cc > 0
    assert np.all(cc[inner] >= 2) and np.all(cc[inner] <= n)
    assert np.all(pc[~inner] >= 1) and np.all(pc[~inner] <= l)
    # every triangle in exactly one leaf
    covered = np.zeros(b.info["n_tris"], np.int64)
    for i in np.nonzero(~inner)[0]:
        covered[c["prim_begin"][i]:c["prim_begin"][i] + pc[i]] += 1
    assert np.all(covered == 1)
    assert sorted(c["prim_ids"].tolist()) == list(range(tris.shape[0]))
    # siblings consecutive, children one level deeper, boxes nested
    lo, hi = c["lo3"], c["hi3"]
    for i in np.nonzero(inner)[0]:
        ch = np.arange(c["child_begin"][i], c["child_begin"][i] + cc[i])
        assert np.all(c["depth"][ch] == c["depth"][i] + 1)
        assert np.all(lo[ch] >= lo[i]) and np.all(hi[ch] <= hi[i])
        # traverseOrderEachAxis: ascending (max + min) + 0.5 centres, ties by index
        for a in range(3):
            o = c["order48"][i, a * 16:a * 16 + cc[i]].astype(int)
            assert sorted(o.tolist()) == list(range(cc[i]))
            cen = (hi[ch, a] + lo[ch, a]) + np.float32(0.5)
            keys = list(zip(cen[o].tolist(), o.tolist()))
            assert keys == sorted(keys)
    # leaf boxes bound their triangles
    pts = c["prim_tri9"].reshape(-1, 3, 3)
    for i in np.nonzero(~inner)[0]:
        p = pts[c["prim_begin"][i]:c["prim_begin"][i] + pc[i]].reshape(-1, 3)
        assert np.all(p.min(0) == lo[i]) and np.all(p.max(0) == hi[i])
    assert b.info["depth"] == int(c["depth"][~inner].max()) + 1
    return c


@pytest.mark.parametrize("n,l", [(4, 4), (8, 8), (16, 16), (12, 4)])
def test_invariants_clutter(n, l):
    tris = S.clutter(40, 2)
    _invariants(pkg.Bvh(tris, n, l), tris)


def test_deterministic():
    tris = S.clutter(40, 2)
    a = pkg.Bvh(tris, 8, 8).export_compact()
    b = pkg.Bvh(tris, 8, 8).export_compact()
    for k in a:
        assert np.array_equal(a[k], b[k])


def test_parallel_build_matches_restatement_on_larger_scene():
    # Large enough that children are built on worker threads.
    tris = S.terrain(110, 9)
    b = pkg.Bvh(tris, 4, 4)
    c = _invariants(b, tris)
    assert b.info["n_tris"] == tris.shape[0] == 24200
    assert c["child_count"][0] >= 2


def test_zero_area_triangles_dropped_ids_kept():
    tris = S.terrain(6, 1)
    deg = np.zeros((2, 9), np.float32)
    mixed = np.concatenate([deg[:1], tris, deg[1:]])
    b = pkg.Bvh(mixed, 4, 4)
    assert b.info["n_tris"] == tris.shape[0]
    ids = b.export_compact()["prim_ids"]
    assert ids.min() == 1 and ids.max() == tris.shape[0]


def test_single_triangle_is_a_root_leaf():
    b = pkg.Bvh(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), 4, 4)
    c = b.export_compact()
    assert b.info["n_nodes"] == 1 and c["prim_count"][0] == 1 and b.info["max_stack"] == 1


def test_max_stack_bound():
    tris = S.clutter(40, 2)
    b = pkg.Bvh(tris, 8, 4)
    c = b.export_compact()
    # 1 + max over root-to-leaf paths of sum(children - 1)
    def extra(i):
        if c["child_count"][i] == 0:
            return 0
        ch = range(c["child_begin"][i], c["child_begin"][i] + c["child_count"][i])
        return int(c["child_count"][i]) - 1 + max(extra(j) for j in ch)
    assert b.info["max_stack"] == 1 + extra(0)


@pytest.mark.parametrize("gang,n,l", [(4, 4, 4), (4, 8, 12), (8, 8, 8), (4, 16, 16), (4, 5, 3)])
def test_fast_export_layout(gang, n, l):
    tris = S.clutter(6, 4)
    b = pkg.Bvh(tris, n, l)
    c = b.export_compact()
    f = b.export_fast(gang=gang)
    nm, lm = f["node_memory"], f["leaf_memory"]
    assert nm == -(-n // gang) * gang and lm == -(-l // gang) * gang
    tp = f["tri_points"]
    for i in range(b.info["n_nodes"]):
        bd = f["bounds"][i]
        if c["child_count"][i] == 0:
            assert np.isnan(bd[0])
            beg = f["begin"][i]
            cnt = int(c["prim_count"][i])
            real = -(-cnt // gang) * gang
            blk = tp[beg:beg + lm * 9]
            if real != lm:
                assert blk[-2] == real and np.isnan(blk[-1])
            pts = c["prim_tri9"][c["prim_begin"][i]:c["prim_begin"][i] + cnt]
            for v in range(3):
                for a in range(3):
                    row = blk[(v * 3 + a) * real:(v * 3 + a) * real + real]
                    assert np.array_equal(row[:cnt], pts[:, v * 3 + a])
                    assert np.all(row[cnt:] == 0)
        else:
            cnt = int(c["child_count"][i])
            real = -(-cnt // gang) * gang
            ch = np.arange(c["child_begin"][i], c["child_begin"][i] + cnt)
            assert f["begin"][i] == c["child_begin"][i]
            for a in range(3):
                assert np.array_equal(bd[a * real:a * real + cnt], c["lo3"][ch, a])
                assert np.array_equal(bd[3 * real + a * real:3 * real + a * real + cnt], c["hi3"][ch, a])
            if real != nm:
                assert bd[-2] == real and np.isnan(bd[-1])
            types = sum(1 << j for j, x in enumerate(ch) if c["child_count"][x] > 0)
            assert f["child_type"][i] == types
            for a in range(3):
                assert np.array_equal(f["order"][i, a * nm:a * nm + cnt], c["order48"][i, a * 16:a * 16 + cnt])
    assert tp.shape[0] == b.info["n_leaves"] * lm * 9


def test_import_compact_round_trip():
    """A tree handed over as CompactNodeV3 arrays (bvhgpu_bvh_import_compact)
    exports the same arrays, FastNodeManager view and device records, with
    the same worst-case stack height."""
    from tests import _scenes as TS
    for n, l in ((4, 4), (8, 8), (16, 4)):
        _, b, _ = TS.bvh("clutter120", n, l)
        c = b.export_compact()
        b2 = pkg.Bvh.from_compact(c, n, l)
        c2 = b2.export_compact()
        for k in c:
            assert np.array_equal(c[k], c2[k]), k
        f, f2 = b.export_fast(), b2.export_fast()
        for k in ("bounds", "begin", "order", "child_type", "tri_points"):
            assert np.array_equal(np.asarray(f[k]).view(np.uint8), np.asarray(f2[k]).view(np.uint8)), k
        for fmt in ("fp32", "q8"):
            assert np.array_equal(b.node_records(node_format=fmt), b2.node_records(node_format=fmt))
        assert b2.info["max_stack"] == b.info["max_stack"]
        assert b2.info["depth"] == b.info["depth"]


def test_import_compact_rejects_bad_trees():
    from tests import _scenes as TS
    _, b, _ = TS.bvh("clutter120", 4, 4)
    c = b.export_compact()
    inner = np.nonzero(c["child_count"] > 0)[0]
    leaf = np.nonzero(c["child_count"] == 0)[0]

    def bad(mut):
        d = {k: v.copy() for k, v in c.items()}
        mut(d)
        with pytest.raises(pkg.BvhgpuError):
            pkg.Bvh.from_compact(d, 4, 4)

    bad(lambda d: d["child_begin"].__setitem__(inner[1], 0))            # child before parent
    bad(lambda d: d["child_begin"].__setitem__(inner[0], len(d["child_count"])))  # out of range
    bad(lambda d: d["order48"].__setitem__((inner[0], 1), d["order48"][inner[0], 0]))  # not a permutation
    bad(lambda d: d["prim_count"].__setitem__(leaf[0], 5))               # leaf above L
    bad(lambda d: d["prim_begin"].__setitem__(leaf[0], len(d["prim_ids"])))  # outside the primitives
    bad(lambda d: d["prim_tri9"].__setitem__((0, 0), np.inf))            # non-finite vertex
