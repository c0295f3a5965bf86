"""ctypes wrapper of the CPU oracle (oracle/bvh_oracle.c) — TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module. Parity status: the instrumented profile is pinned
against the reference's own code compiled here (oracle/ref/) and the fixtures
it generated (tests/golden/); the fast (ISPC) profile is not, see the header
of bvh_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from .build_oracle import build, build_baseline

_P = C.c_void_p


class _Compact(C.Structure):
    _fields_ = [("n_nodes", C.c_uint64)] + [(k, _P) for k in (
        "lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "order48",
        "depth", "prim_ids", "prim_tri9")]


class _Fast(C.Structure):
    _fields_ = [("n_nodes", C.c_uint64), ("gang", C.c_int32), ("node_memory", C.c_int32),
                ("leaf_memory", C.c_int32)] + [(k, _P) for k in (
                    "bounds", "begin", "order", "child_type", "tri_points")]


_lib = None
_blib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """The scalar oracle library."""
    global _lib
    with _lock:
        if _lib is None:
            _lib = _bind(C.CDLL(str(build())))
    return _lib


def baseline_lib() -> C.CDLL:
    """The vectorised build of the same source, timed as the CPU baseline."""
    global _blib
    with _lock:
        if _blib is None:
            _blib = _bind(C.CDLL(str(build_baseline())))
    return _blib


def _bind(L: C.CDLL) -> C.CDLL:
    L.oracle_trace_instrumented.restype = C.c_int
    L.oracle_trace_instrumented.argtypes = [C.POINTER(_Compact), _P, C.c_uint64, C.c_int,
                                            _P, _P, _P, _P, C.c_int, _P]
    L.oracle_trace_instrumented_stream.restype = C.c_int
    L.oracle_trace_instrumented_stream.argtypes = [C.POINTER(_Compact), _P, C.c_uint64,
                                                   C.c_int, C.c_int, _P, _P, _P, _P, _P]
    L.oracle_trace_instrumented_stream_steps.restype = C.c_int
    L.oracle_trace_instrumented_stream_steps.argtypes = [
        C.POINTER(_Compact), _P, C.c_uint64, C.c_int, C.c_int, _P, _P, _P, _P, C.c_int,
        _P, _P, C.c_int, _P]
    L.oracle_trace_fast.restype = C.c_int
    L.oracle_trace_fast.argtypes = [C.POINTER(_Fast), C.POINTER(_Compact), _P, C.c_uint64,
                                    C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P,
                                    C.c_int]
    L.oracle_hit_points.restype = None
    L.oracle_hit_points.argtypes = [_P, _P, C.c_uint64, _P]
    L.oracle_fp64_pairs.restype = None
    L.oracle_fp64_pairs.argtypes = [_P, _P, C.c_uint64, C.c_int, _P]
    L.oracle_aabb_intersect_calls.restype = None
    L.oracle_aabb_intersect_calls.argtypes = [C.c_int32, _P, _P, _P, _P, _P, C.c_uint64]
    L.oracle_tri_intersect_calls.restype = None
    L.oracle_tri_intersect_calls.argtypes = [C.c_int32, C.c_int32, _P, _P, _P, _P,
                                             C.c_uint64]
    L.oracle_tri_any_hit_calls.restype = None
    L.oracle_tri_any_hit_calls.argtypes = [C.c_int32, _P, _P, _P, _P, C.c_uint64]
    return L


def _p(a):
    return None if a is None else a.ctypes.data


class CompactView:
    """Keeps the exported CompactNodeV3 arrays alive next to the C view."""

    def __init__(self, arrays: dict):
        self.a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
        self.c = _Compact(self.a["child_count"].shape[0], *[_p(self.a[k]) for k in (
            "lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "order48",
            "depth", "prim_ids", "prim_tri9")])


class FastView:
    def __init__(self, arrays: dict):
        self.a = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v)
                  for k, v in arrays.items()}
        self.c = _Fast(self.a["begin"].shape[0], self.a["gang"], self.a["node_memory"],
                       self.a["leaf_memory"], *[_p(self.a[k]) for k in (
                           "bounds", "begin", "order", "child_type", "tri_points")])


def trace_instrumented(view: CompactView, rays: np.ndarray, shadow: bool, packet: int = 0,
                       counters: bool = True, use_distance: bool = False) -> dict:
    """CompactNodeManager::intersectImmediately(ray, use_distance) (packet ==
    0) or intersectWideAlternative over packets of ``packet`` rays. With
    ``counters``: per-ray counters, per-depth node / leaf visits
    (``depth_hist``) and Ray::childFullness / primitiveFullness summed over
    the rays (``fullness`` [2, 17]: visits of nodes with c children, of leaves
    with c triangles)."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    hits = None if shadow else np.zeros((n, 4), np.float32)
    occ = np.zeros(n, np.uint8) if shadow else None
    ctr = np.zeros((n, 8), np.uint32) if counters else None
    hist = np.zeros((2, 64), np.uint64) if counters else None
    full = np.zeros((2, 17), np.uint64) if counters else None
    if packet and use_distance:
        raise ValueError("use_distance is a per-ray traversal")
    if packet:
        rc = lib().oracle_trace_instrumented_stream(C.byref(view.c), _p(rays), n, int(shadow),
                                                     packet, _p(hits), _p(occ), _p(ctr), _p(hist),
                                                     _p(full))
    else:
        rc = lib().oracle_trace_instrumented(C.byref(view.c), _p(rays), n, int(shadow), _p(hits),
                                             _p(occ), _p(ctr), _p(hist), int(use_distance),
                                             _p(full))
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return {"hits": hits, "occluded": occ, "counters": ctr, "depth_hist": hist, "fullness": full}


def trace_fast(fview: FastView, cview: CompactView, rays: np.ndarray, any_hit: bool,
               packet: int = 0, threads: int = 0, counters: bool = True,
               outputs: bool = True, use_distance: bool = False, baseline: bool = False) -> dict:
    """FastNodeManager::intersect / intersectSecondary (packet == 0) or the
    WideAlternative stream versions, with ISPC gang-lane semantics;
    ``use_distance``: intersectSaveDistance (per ray). ``baseline``: the
    vectorised build (libcpubaseline.so), the timed CPU baseline."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    hits = np.zeros((n, 4), np.float32) if (outputs and not any_hit) else None
    occ = np.zeros(n, np.uint8) if (outputs and any_hit) else None
    li = np.zeros(n, np.int32) if (outputs and not any_hit) else None
    ti = np.zeros(n, np.int8) if (outputs and not any_hit) else None
    ctr = np.zeros((n, 8), np.uint32) if counters else None
    hist = np.zeros((2, 64), np.uint64) if counters else None
    L = baseline_lib() if baseline else lib()
    rc = L.oracle_trace_fast(C.byref(fview.c), C.byref(cview.c), _p(rays), n, int(any_hit),
                                 packet, threads, _p(hits), _p(occ), _p(li), _p(ti), _p(ctr),
                                 _p(hist), int(use_distance))
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return {"hits": hits, "occluded": occ, "leaf_index": li, "tri_index": ti, "counters": ctr,
            "depth_hist": hist}


def trace_instrumented_steps(view: CompactView, rays: np.ndarray, shadow: bool, packet: int,
                             step_cap: int, wide_alternative: bool = True) -> dict:
    """intersectWideAlternative over packets of ``packet`` rays with the
    per-step workgroup data (bvh_oracle.c: stream_impl): ``steps`` [packets,
    step_cap, 5] (node work, unique nodes, leaf work, unique leaves,
    terminations) and ``step_count`` [packets], plus hits / occlusion and
    counters."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    npk = -(-n // packet)
    hits = None if shadow else np.zeros((n, 4), np.float32)
    occ = np.zeros(n, np.uint8) if shadow else None
    ctr = np.zeros((n, 8), np.uint32)
    hist = np.zeros((2, 64), np.uint64)
    steps = np.zeros((npk, step_cap, 5), np.uint32)
    count = np.zeros(npk, np.uint32)
    full = np.zeros((2, 17), np.uint64)
    rc = lib().oracle_trace_instrumented_stream_steps(
        C.byref(view.c), _p(rays), n, int(shadow), packet, _p(hits), _p(occ), _p(ctr), _p(hist),
        step_cap, _p(steps), _p(count), int(wide_alternative), _p(full))
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return {"hits": hits, "occluded": occ, "counters": ctr, "depth_hist": hist, "steps": steps,
            "step_count": count, "fullness": full}


def hit_points(rays: np.ndarray, tri9: np.ndarray) -> np.ndarray:
    """Triangle::intersect's hit point b0 p0 + b1 p1 + b2 p2 of each (ray,
    triangle) pair, instrumented profile (NaN where the pair does not hit)."""
    rays = np.ascontiguousarray(rays, np.float32)
    tri9 = np.ascontiguousarray(tri9, np.float32)
    out = np.zeros((rays.shape[0], 3), np.float32)
    lib().oracle_hit_points(_p(rays), _p(tri9), rays.shape[0], _p(out))
    return out


def fp64_pairs(rays: np.ndarray, tri9: np.ndarray, normalise: bool) -> np.ndarray:
    """Double-precision (t, b1, b2) of each (ray, triangle) pair."""
    rays = np.ascontiguousarray(rays, np.float32)
    tri9 = np.ascontiguousarray(tri9, np.float32)
    out = np.zeros((rays.shape[0], 3), np.float64)
    lib().oracle_fp64_pairs(_p(rays), _p(tri9), rays.shape[0], int(normalise), _p(out))
    return out


def aabb_intersect_calls(n: int, bounds: np.ndarray, offsets: np.ndarray, fastrays: np.ndarray,
                         distances: np.ndarray):
    """aabbIntersect{n} per call (bvh_oracle.c: oracle_aabb_intersect_calls):
    returns (result [count] u8, distances [count, n] with t0 written at hit
    lanes of the given array)."""
    bounds = np.ascontiguousarray(bounds, np.float32)
    offsets = np.ascontiguousarray(offsets, np.uint32)
    fastrays = np.ascontiguousarray(fastrays, np.float32)
    dist = np.array(distances, np.float32, copy=True, order="C")
    res = np.zeros(offsets.shape[0], np.uint8)
    lib().oracle_aabb_intersect_calls(n, _p(bounds), _p(offsets), _p(fastrays), _p(dist),
                                      _p(res), offsets.shape[0])
    return res, dist


def tri_intersect_calls(l: int, gang: int, tri: np.ndarray, ids: np.ndarray,
                        fastrays: np.ndarray):
    """triIntersect{l} per call: returns (in-leaf index or -1, the FastRay
    records with tMax lowered on hits)."""
    tri = np.ascontiguousarray(tri, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    fr = np.array(fastrays, np.float32, copy=True, order="C")
    res = np.zeros(ids.shape[0], np.int32)
    lib().oracle_tri_intersect_calls(l, gang, _p(tri), _p(ids), _p(fr), _p(res), ids.shape[0])
    return res, fr


def tri_any_hit_calls(l: int, tri: np.ndarray, ids: np.ndarray, fastrays: np.ndarray):
    """triAnyHit{l} per call: returns [count] u8."""
    tri = np.ascontiguousarray(tri, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    fr = np.ascontiguousarray(fastrays, np.float32)
    res = np.zeros(ids.shape[0], np.uint8)
    lib().oracle_tri_any_hit_calls(l, _p(tri), _p(ids), _p(fr), _p(res), ids.shape[0])
    return res


class _Tree(C.Structure):
    _fields_ = [("n_nodes", C.c_uint64), ("n_prims", C.c_uint64), ("depth", C.c_int32),
                ("max_stack", C.c_int32)] + [(k, _P) for k in (
                    "lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count",
                    "order48", "depth_of", "prim_ids", "prim_tri9")]


# The reference's SSE SAH factor table (sahFactorConfigSse.txt, read by
# RayTracer::loadSahFactor, rayTracer.cpp:880-925): rows node size 4..16,
# columns leaf size 4..16 after rounding both up to the gang of 4; gang 8
# (the AVX table) gives 1. Decimal text as float32 (std::stof).
_SAH_SSE = ((0.9790158394920848, 0.6019200777645688, 0.46148535855892625, 0.38099865799955585),
            (1.3129201663140904, 0.8089449478051558, 0.6356877674077516, 0.5431092069456159),
            (1.5611955563121058, 0.9667477491937599, 0.7477536713402126, 0.638505587529224),
            (1.8033700927282266, 1.1369639789217003, 0.8735301252614894, 0.7655054621988963))


def sah_factor(branching: int, leaf_size: int, gang: int = 4) -> float:
    if gang == 8:
        return 1.0
    tn = -(-branching // gang) * gang
    tl = -(-leaf_size // gang) * gang
    if not (4 <= tn <= 16 and 4 <= tl <= 16):
        return 1.0
    return float(np.float32(_SAH_SSE[tn // 4 - 1][tl // 4 - 1]))


def build_tree(tris, branching: int, leaf_size: int, *, leaf_split_option: int = 1,
               sah: float | None = None, gang: int = 4) -> dict:
    """The reference's SAH tree of world-space triangles ``[T, 9]``
    (oracle/sah_builder.c), as CompactNodeV3 arrays in the layout of
    ``bvhraytracer_gb300.Bvh.export_compact``, plus ``depth_levels`` and
    ``max_stack``."""
    t9 = np.ascontiguousarray(np.asarray(tris, np.float32).reshape(-1, 9))
    L = lib()
    if not hasattr(L, "_tree_bound"):
        L.oracle_build_tree.restype = C.c_int
        L.oracle_build_tree.argtypes = [_P, C.c_uint64, C.c_int32, C.c_int32, C.c_int32,
                                        C.c_float, C.POINTER(_Tree)]
        L.oracle_tree_free.restype = None
        L.oracle_tree_free.argtypes = [C.POINTER(_Tree)]
        L._tree_bound = True
    tr = _Tree()
    f = sah_factor(branching, leaf_size, gang) if sah is None else float(sah)
    rc = L.oracle_build_tree(_p(t9), t9.shape[0], branching, leaf_size, leaf_split_option, f,
                             C.byref(tr))
    if rc:
        raise RuntimeError(f"oracle tree build failed ({rc})")
    try:
        n, m = tr.n_nodes, tr.n_prims

        def arr(ptr, ctype, count, dtype):
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), (count,)).astype(
                dtype, copy=True)

        out = {"lo3": arr(tr.lo3, C.c_float, 3 * n, np.float32).reshape(n, 3),
               "hi3": arr(tr.hi3, C.c_float, 3 * n, np.float32).reshape(n, 3),
               "child_begin": arr(tr.child_begin, C.c_uint32, n, np.uint32),
               "child_count": arr(tr.child_count, C.c_uint32, n, np.uint32),
               "prim_begin": arr(tr.prim_begin, C.c_uint32, n, np.uint32),
               "prim_count": arr(tr.prim_count, C.c_uint32, n, np.uint32),
               "order48": arr(tr.order48, C.c_int8, 48 * n, np.int8).reshape(n, 48),
               "depth": arr(tr.depth_of, C.c_uint8, n, np.uint8),
               "prim_ids": arr(tr.prim_ids, C.c_uint32, m, np.uint32),
               "prim_tri9": arr(tr.prim_tri9, C.c_float, 9 * m, np.float32).reshape(m, 9),
               "depth_levels": int(tr.depth), "max_stack": int(tr.max_stack)}
    finally:
        L.oracle_tree_free(C.byref(tr))
    return out


def fast_arrays(tree: dict, gang: int = 4, node_memory: int = 0, leaf_memory: int = 0) -> dict:
    """FastNodeManager's flat arrays (fastNodeManager.h:1495-1688) from
    CompactNodeV3 arrays (``build_tree``): per node the children's bounds as
    SoA rows of the gang-rounded child count (a (count, NaN) sentinel in the
    last two floats when that is below the node memory), the first child id,
    the per-axis push sequences and the inner-child bit mask; per leaf a
    ``trianglePoints`` block of 9 rows, each the gang-rounded triangle count
    long, in a 9 x leaf-memory slot with the same kind of sentinel, and
    ``begin`` = the block's float offset (the hit encoding's leafIndex); a
    leaf's bounds[0] is NaN. The layout ``FastView`` reads."""
    cc = tree["child_count"].astype(np.int64)
    pc = tree["prim_count"].astype(np.int64)
    n = cc.shape[0]
    nm = node_memory or -(-int(cc.max()) // gang) * gang
    lm = leaf_memory or -(-int(pc.max()) // gang) * gang
    nan = np.float32(np.nan)
    bounds = np.zeros((n, 6 * nm), np.float32)
    order = np.zeros((n, 3 * nm), np.int8)
    begin = np.zeros(n, np.uint32)
    child_type = np.zeros(n, np.uint32)
    inner = np.nonzero(cc > 0)[0]
    real = (-(-cc // gang)) * gang
    # children of inner nodes: (node, slot j)
    rep = np.repeat(inner, cc[inner])
    j = np.arange(rep.shape[0]) - np.repeat(np.cumsum(cc[inner]) - cc[inner], cc[inner])
    child = tree["child_begin"][rep].astype(np.int64) + j
    r = real[rep]
    for i in range(3):
        bounds[rep, i * r + j] = tree["lo3"][child, i]
        bounds[rep, 3 * r + i * r + j] = tree["hi3"][child, i]
    sent = inner[real[inner] != nm]
    bounds[sent, 6 * nm - 2] = real[sent].astype(np.float32)
    bounds[sent, 6 * nm - 1] = nan
    is_inner_child = (cc[child] > 0).astype(np.uint32)
    np.bitwise_or.at(child_type, rep, is_inner_child << j.astype(np.uint32))
    begin[inner] = tree["child_begin"][inner]
    o48 = tree["order48"].reshape(n, 3, 16)
    for a in range(3):
        order[rep, a * nm + j] = o48[rep, a, j]
    # leaf blocks, in node order
    leaves = np.nonzero(pc > 0)[0]
    tri = np.zeros((leaves.shape[0], 9 * lm), np.float32)
    lrep = np.repeat(np.arange(leaves.shape[0]), pc[leaves])
    k = np.arange(lrep.shape[0]) - np.repeat(np.cumsum(pc[leaves]) - pc[leaves], pc[leaves])
    lreal = (-(-pc // gang)) * gang
    rl = lreal[leaves][lrep]
    slot = tree["prim_begin"][leaves][lrep].astype(np.int64) + k
    for row in range(9):  # rows x0 y0 z0 x1 ... z2
        tri[lrep, row * rl + k] = tree["prim_tri9"][slot, row]
    lsent = np.nonzero(lreal[leaves] != lm)[0]
    tri[lsent, 9 * lm - 2] = lreal[leaves][lsent].astype(np.float32)
    tri[lsent, 9 * lm - 1] = nan
    begin[leaves] = (np.arange(leaves.shape[0]) * 9 * lm).astype(np.uint32)
    bounds[leaves, 0] = nan
    return {"bounds": bounds, "begin": begin, "order": order, "child_type": child_type,
            "tri_points": tri.reshape(-1), "gang": gang, "node_memory": nm, "leaf_memory": lm}
