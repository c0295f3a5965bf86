"""Pure-Python restatement of the reference's SAH builder — TEST INFRASTRUCTURE.

Independent of the C++ builder in libbvhgpu.so; the CPU tests compare the two
node for node on small scenes. Float arithmetic uses numpy float32 scalars
(IEEE single, no fused multiply-add), in the reference's evaluation order:

  chooseAxisAndSort ............. src/accelerationStructure/aabb.h:40-67
  Aabb::calculateBounds / SA .... aabb.h:113-134
  Node::sah (step variant c) .... src/accelerationStructure/node.h:66-91
  computerBestSplit[Sort] ....... src/accelerationStructure/aabb.cpp:4-69
  Aabb::recursiveBvh ............ aabb.cpp:71-206
  calculateTraverseOrderEachAxis  src/accelerationStructure/node.cpp:254-275
  customTreeOrder ............... src/accelerationStructure/compactNode.cpp:997-1008

Sorting is stable (the reference's parallel sort leaves equal centres in an
unspecified order). Pure-Python loops: small scenes only.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def _min(a, b):
    return b if b < a else a


def _max(a, b):
    return b if a < b else a


def _max_dim(v):
    return (0 if v[0] > v[2] else 2) if v[0] > v[1] else (1 if v[1] > v[2] else 2)


class _Node:
    __slots__ = ("lo", "hi", "begin", "end", "depth", "children", "order")

    def __init__(self):
        self.children = []
        self.order = [[], [], []]


def build(tris: np.ndarray, branching: int, leaf_size: int, sah_factor: float,
          leaf_split_option: int = 1) -> dict:
    """Builds the tree; returns the CompactNodeV3 view as numpy arrays in the
    layout of ``Bvh.export_compact`` (zero-area triangles must be removed by
    the caller)."""
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    T = tris.shape[0]
    bmin = [[None] * 3 for _ in range(T)]
    bmax = [[None] * 3 for _ in range(T)]
    cen = [[None] * 3 for _ in range(T)]
    for i in range(T):
        for k in range(3):
            p0, p1, p2 = f32(tris[i, 0, k]), f32(tris[i, 1, k]), f32(tris[i, 2, k])
            lo = _min(_min(p0, p1), p2)
            hi = _max(_max(p0, p1), p2)
            bmin[i][k], bmax[i][k] = lo, hi
            cen[i][k] = hi * f32(0.5) + lo * f32(0.5)
    prims = list(range(T))
    sah_factor = f32(sah_factor)
    L = leaf_size
    N = branching

    def sort_range(b, e):
        mn = [f32(222222.0)] * 3
        mx = [f32(-222222.0)] * 3
        for i in range(b, e):
            c = cen[prims[i]]
            for k in range(3):
                mn[k] = _min(mn[k], c[k])
                mx[k] = _max(mx[k], c[k])
        axis = _max_dim([mx[k] - mn[k] for k in range(3)])
        seg = prims[b:e]
        seg.sort(key=lambda p: cen[p][axis])  # stable
        prims[b:e] = seg
        return axis

    def area(lo, hi):
        dx, dy, dz = hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]
        return f32(2.0) * (dx * dy + dx * dz + dy * dz)

    def sah(count, lo, hi, inv_area):
        steps = (count - 1) // L + 1
        return f32(steps) * area(lo, hi) * inv_area * f32(L)

    def best_split(b, e, inv_area):
        sort_range(b, e)
        size = e - b
        metric = [f32(0.0)] * (size - 1)
        lo = [f32(222222.0)] * 3
        hi = [f32(-222222.0)] * 3
        for j in range(size - 1):
            p = prims[b + j + 1]  # Node::sweepRight reads the element at the new end
            lo = [_min(lo[k], bmin[p][k]) for k in range(3)]
            hi = [_max(hi[k], bmax[p][k]) for k in range(3)]
            metric[j] = metric[j] + sah(j + 1, lo, hi, inv_area)
        lo = [f32(222222.0)] * 3
        hi = [f32(-222222.0)] * 3
        for j in range(size - 2, -1, -1):
            p = prims[b + j + 1]
            lo = [_min(lo[k], bmin[p][k]) for k in range(3)]
            hi = [_max(hi[k], bmax[p][k]) for k in range(3)]
            metric[j] = metric[j] + sah(size - 1 - j, lo, hi, inv_area)
        best = 0
        for j in range(1, len(metric)):
            if metric[j] < metric[best]:
                best = j
        return b + best + 1, metric[best]

    def bounds(n):
        lo = [f32(222222.0)] * 3
        hi = [f32(-222222.0)] * 3
        for i in range(n.begin, n.end):
            p = prims[i]
            lo = [_min(lo[k], bmin[p][k]) for k in range(3)]
            hi = [_max(hi[k], bmax[p][k]) for k in range(3)]
        n.lo, n.hi = lo, hi

    def recurse(n):
        count = n.end - n.begin
        if count <= L and leaf_split_option in (0, 2):
            return
        sort_range(n.begin, n.end)
        work = [[n.begin, n.end]]
        best_i = 0
        inv_area = f32(1.0) / area(n.lo, n.hi)
        for _ in range(N - 1):
            pc = 0
            for i, w in enumerate(work):
                if pc < w[1] - w[0]:
                    pc = w[1] - w[0]
                    best_i = i
            if pc <= L:
                break
            s, _c = best_split(work[best_i][0], work[best_i][1], inv_area)
            p2 = [s, work[best_i][1]]
            work[best_i][1] = s
            work.insert(best_i + 1, p2)
        if leaf_split_option in (1, 2):
            b = len(work) - 1
            while b < N - 1:
                best_imp = f32(0.0)
                best_id = -1
                best_at = 0
                for i, w in enumerate(work):
                    cnt = w[1] - w[0]
                    if cnt == 1:
                        continue
                    leaf_cost = f32(cnt)
                    s, split_cost = best_split(w[0], w[1], inv_area)
                    split_cost = split_cost + sah_factor
                    if leaf_cost - split_cost > best_imp:
                        best_imp = leaf_cost - split_cost
                        best_id = i
                        best_at = s
                if best_imp == 0:
                    break
                p2 = [best_at, work[best_id][1]]
                work[best_id][1] = best_at
                work.insert(best_id + 1, p2)
                b += 1
        if len(work) == 1:
            return
        for w in work:
            c = _Node()
            c.begin, c.end, c.depth = w[0], w[1], n.depth + 1
            bounds(c)
            n.children.append(c)
        for face in range(3):
            tup = sorted(((c.hi[face] + c.lo[face]) + f32(0.5), i) for i, c in enumerate(n.children))
            n.order[face] = [i for _, i in tup]
        n.begin = n.end
        for c in n.children:
            recurse(c)

    sort_range(0, T)  # RayTracer::preparePrimitives
    root = _Node()
    root.begin, root.end, root.depth = 0, T, 0
    bounds(root)
    recurse(root)

    order = [root]

    def custom(n):
        for c in n.children:
            order.append(c)
        for c in n.children:
            custom(c)

    custom(root)
    ids = {id(n): i for i, n in enumerate(order)}
    nn = len(order)
    out = {
        "lo3": np.zeros((nn, 3), np.float32), "hi3": np.zeros((nn, 3), np.float32),
        "child_begin": np.zeros(nn, np.uint32), "child_count": np.zeros(nn, np.uint32),
        "prim_begin": np.zeros(nn, np.uint32), "prim_count": np.zeros(nn, np.uint32),
        "order48": np.zeros((nn, 48), np.int8), "depth": np.zeros(nn, np.uint8),
        "prim_ids": np.array(prims, np.uint32),
    }
    for i, n in enumerate(order):
        out["lo3"][i] = n.lo
        out["hi3"][i] = n.hi
        out["depth"][i] = n.depth
        if n.children:
            out["child_begin"][i] = ids[id(n.children[0])]
            out["child_count"][i] = len(n.children)
            for a in range(3):
                out["order48"][i, a * 16:a * 16 + len(n.order[a])] = n.order[a]
        else:
            out["prim_begin"][i] = n.begin
            out["prim_count"][i] = n.end - n.begin
    return out
